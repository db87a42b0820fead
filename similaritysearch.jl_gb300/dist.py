"""Distance types accepted by the GPU index (mirror of SimilaritySearch.jl ``Dist``).

Only the distances on the exhaustive path exist here; each carries the
metric code of include/ssgpu.h.  ``evaluate`` is a small host helper for
single pairs (the reference's ``Dist.evaluate``); the bulk work runs on the GPU.
"""
from __future__ import annotations

import numpy as np

from . import _native as N


class PreMetric:
    code: int = -1
    cast_f32: bool = False
    name: str = "PreMetric"

    def __repr__(self):
        return self.name + "()"

    def __eq__(self, other):
        return type(self) is type(other)

    def __hash__(self):
        return hash(type(self))


class SqL2(PreMetric):
    """sum (a_i - b_i)^2  -- src/dist/vecs.jl:86,93-102"""
    code, name = N.METRIC_SQL2, "SqL2"


class L2(PreMetric):
    """sqrt(sum (a_i - b_i)^2)  -- src/dist/vecs.jl:52,59-67"""
    code, name = N.METRIC_L2, "L2"


class NormCosine(PreMetric):
    """1 - sum a_i b_i for normalised vectors  -- src/dist/cos.jl:39,76-84"""
    code, name = N.METRIC_NORMCOSINE, "NormCosine"


class Cosine(PreMetric):
    """1 - dot(a, b) / (norm(a) norm(b))  -- src/dist/cos.jl:16,103"""
    code, name = N.METRIC_COSINE, "Cosine"


class InnerProduct(PreMetric):
    """-dot(a, b): maximum-inner-product ranking (NormCosine minus one; no
    reference type exists -- the reference ranks MIPS with NormCosine on
    unnormalised data, src/dist/cos.jl:78-84)."""
    code, name = N.METRIC_IP, "InnerProduct"


class _Bits:
    class Hamming(PreMetric):
        """Float32(sum count_ones(a_w xor b_w)) over UInt64 words -- src/dist/bits.jl:10,18-25"""
        code, name = N.METRIC_HAMMING, "Bits.Hamming"


class _CastF32:
    """Float32-casting twins (src/dist/vecs-cast-f32.jl): any numeric element
    type is cast to Float32 element by element before the sum."""

    class SqL2(SqL2):
        cast_f32, name = True, "CastF32.SqL2"

    class L2(L2):
        cast_f32, name = True, "CastF32.L2"

    class NormCosine(NormCosine):
        cast_f32, name = True, "CastF32.NormCosine"

    class Cosine(Cosine):
        cast_f32, name = True, "CastF32.Cosine"


class Dist:
    SqL2 = SqL2
    L2 = L2
    NormCosine = NormCosine
    Cosine = Cosine
    InnerProduct = InnerProduct
    Bits = _Bits
    CastF32 = _CastF32


def evaluate(dist: PreMetric, a, b) -> np.float32:
    """Host evaluation of one pair in the reference's formula (index order,
    one fused multiply-add per element is not available in numpy, so this is
    a convenience for examples, not the parity oracle)."""
    if dist.code == N.METRIC_HAMMING:
        a = np.asarray(a, dtype=np.uint64)
        b = np.asarray(b, dtype=np.uint64)
        return np.float32(sum(bin(int(x) ^ int(y)).count("1") for x, y in zip(a.ravel(), b.ravel())))
    a = np.asarray(a, dtype=np.float32).ravel()
    b = np.asarray(b, dtype=np.float32).ravel()
    if dist.code in (N.METRIC_SQL2, N.METRIC_L2):
        d = np.float32(np.sum((a - b) ** 2, dtype=np.float32))
        return np.sqrt(d) if dist.code == N.METRIC_L2 else d
    dot = np.float32(np.dot(a, b))
    if dist.code == N.METRIC_NORMCOSINE:
        return np.float32(1) - dot
    if dist.code == N.METRIC_IP:
        return -dot
    return np.float32(1) - dot / (np.float32(np.linalg.norm(a)) * np.float32(np.linalg.norm(b)))
