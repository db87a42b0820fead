"""similaritysearch_gb300 -- GB300-native exhaustive k-NN behind SimilaritySearch.jl's API.

Host-side mirror of the reference's ``searchbatch`` / ``allknn`` path over a
GPU index (``GPUExhaustiveSearch``) whose work is done by libssgpu.so, the
sm_103a CUDA library with the C ABI of ``include/ssgpu.h``.
"""
from . import _native, shard
from .proj import bitsketch
from .neardup import neardup
from .db import (AbstractDatabase, MatrixDatabase, MMapMatrixDatabase, SubDatabase, VectorDatabase,
                 write_mmap_matrix)
from .dist import Dist, PreMetric, evaluate
from .index import (ArgumentError, GenericContext, GPUExhaustiveSearch, add_distance_evaluations,
                    allknn, allknn_b, append_items_b, database, distance, distance_evaluations, index_b,
                    push_item_b, rerank_b, search, searchbatch, searchbatch_b, searchbatches,
                    bichromatic_closestpair, bichromatic_kclosestpairs, closestpair, closestpairs)
from .log import LOG, InformativeLog, LogList, RecorderLog
from .perf import macrorecall, recallscore
from .pqueue import AbstractKnnQueue, AbstractMetricQueue, AbstractRadiusQueue, IdDist, KnnSorted, RadiusSorted, knnqueue

# ParallelExhaustiveSearch and ExhaustiveSearch return the same results; on the
# GPU both are the same index.
GPUParallelExhaustiveSearch = GPUExhaustiveSearch

__all__ = [
    "AbstractDatabase", "MatrixDatabase", "MMapMatrixDatabase", "SubDatabase", "VectorDatabase", "write_mmap_matrix", "Dist", "PreMetric", "evaluate",
    "ArgumentError", "GenericContext", "GPUExhaustiveSearch", "GPUParallelExhaustiveSearch",
    "add_distance_evaluations", "allknn", "allknn_b", "append_items_b", "database", "distance",
    "distance_evaluations", "index_b", "push_item_b", "rerank_b", "search", "searchbatch",
    "searchbatch_b", "searchbatches", "bichromatic_closestpair", "bichromatic_kclosestpairs", "closestpair",
    "closestpairs", "neardup", "LOG", "InformativeLog", "LogList", "RecorderLog", "macrorecall", "recallscore",
    "IdDist", "KnnSorted", "knnqueue", "bitsketch", "AbstractMetricQueue", "AbstractKnnQueue",
    "AbstractRadiusQueue", "RadiusSorted",
]


def build(verbose: bool = False) -> str:
    """Compiles libssgpu.so in-tree (nvcc, sm_103a)."""
    from .builder import build as _build
    return _build(verbose=verbose)
