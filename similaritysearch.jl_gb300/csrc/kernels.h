// kernels.h -- host-side launchers of the device kernels (internal to libssgpu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ssg {

enum Metric { SQL2 = 0, L2 = 1, NORMCOSINE = 2, COSINE = 3, IP = 4, HAMMING = 5 };

// A scan over database rows [0, n) for m queries.  Each (query, split) pair
// leaves its `kk` smallest keys, sorted ascending, in
// cand[(q * splits + s) * kk + i]; empty slots hold KEY_EMPTY.
struct ScanArgs {
    int metric;
    int64_t n;         // database rows
    int64_t dim;       // floats per row (float metrics) or words (Hamming)
    int64_t m;         // queries
    int kk;            // keys kept per (query, split)
    int splits;        // database splits
    int64_t split_len; // rows per split (last may be shorter)
    uint64_t *cand;    // m * splits * kk keys
    uint64_t *gheap;   // global heap storage when kk is too large for shared memory
    int64_t id_base;   // added to every 0-based row id in the keys
};

// Exact FP32 scan: difference form for SqL2/L2, sequential-FMA dot for the
// others, summed in index order (bit-identical to the oracle's lanes=1 sum).
cudaError_t launch_direct_f32(const ScanArgs &a, const float *db, const float *db_norm,
                              const float *q, const float *q_norm, cudaStream_t st, int *launches);

// Hamming scan over packed UInt64 sketches.
cudaError_t launch_hamming(const ScanArgs &a, const uint64_t *db, const uint64_t *q,
                           cudaStream_t st, int *launches);

// Global-heap bytes a scan needs (0 when its heaps fit in shared memory).
size_t direct_gheap_bytes(const ScanArgs &a);
size_t hamming_gheap_bytes(const ScanArgs &a);

// Merges the `segs` sorted key lists of every query and writes the k
// outputs: 1-based ids and distances, 0 / +Inf when empty.  With
// exclude_self, query j is object j + self_base and is dropped from its list
// (the list holds k+1 keys then).
struct FinalizeArgs {
    const uint64_t *cand;
    int segs;
    int kk;
    int64_t m;
    int k_out;
    int exclude_self;
    int64_t self_base;
    uint32_t *out_ids;
    float *out_dists;
};
cudaError_t launch_finalize(const FinalizeArgs &a, cudaStream_t st, int *launches);

// Row norms: out[i] = sqrt(sum x^2) (COSINE) in sequential FMA order.
cudaError_t launch_row_norms(const float *x, int64_t rows, int64_t dim, float *out,
                             cudaStream_t st, int *launches);

// Element casts to Float32 (CastF32 twins): elem is SSG_ELEM_*.
cudaError_t launch_cast_f32(const void *src, int elem, int64_t count, float *dst,
                            cudaStream_t st, int *launches);

// Exact rerank of candidate id lists (rerank!): per query j, ids[j*len ..]
// (1-based, 0 terminates) are re-scored and sorted by (distance, id).
// db / q are float rows (float metrics) or UInt64 words (HAMMING); norms are
// used by COSINE only.
cudaError_t launch_rerank(int metric, const void *db, const float *db_norm, int64_t dim,
                          const void *q, const float *q_norm, int64_t m, int len,
                          uint32_t *ids, float *dists, cudaStream_t st, int *launches);

int device_sm_count();

}  // namespace ssg
