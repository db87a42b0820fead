// rerank.cu -- exact re-scoring of candidate lists (rerank!, src/rerank.jl:22-41).
//
// For query j, the ids in row j (1-based; the first 0 ends the list, as in
// the reference) are re-evaluated with the exact distance and the valid prefix
// is sorted.  The reference sorts with sortperm and leaves the order of equal
// distances to Base.sort; here ties are ordered by id, which is one of the
// orders the reference can produce and makes the output deterministic.
#include "common.cuh"
#include "kernels.h"

namespace ssg {

namespace {

// Exact distance of one (row, query) pair, summed in index order with one FMA
// per element -- the same chain as the scan kernels and the oracle.
template <int METRIC>
__device__ float exact_pair(const void *dbv, int64_t row, int64_t dim, const void *qv, int64_t j,
                            const float *xn, const float *qn) {
    if (METRIC == HAMMING) {
        const uint64_t *x = static_cast<const uint64_t *>(dbv) + row * dim;
        const uint64_t *q = static_cast<const uint64_t *>(qv) + j * dim;
        int d = 0;
        for (int64_t w = 0; w < dim; ++w) d += __popcll(x[w] ^ q[w]);
        return float(d);
    }
    const float *x = static_cast<const float *>(dbv) + row * dim;
    const float *q = static_cast<const float *>(qv) + j * dim;
    float acc = 0.0f;
    if (METRIC == SQL2 || METRIC == L2) {
        for (int64_t c = 0; c < dim; ++c) { float m = x[c] - q[c]; acc = fmaf(m, m, acc); }
        return METRIC == L2 ? sqrtf(acc) : acc;
    }
    for (int64_t c = 0; c < dim; ++c) acc = fmaf(x[c], q[c], acc);
    if (METRIC == NORMCOSINE) return 1.0f - acc;
    if (METRIC == IP) return -acc;
    return 1.0f - acc / (xn[row] * qn[j]);
}

template <int METRIC>
__global__ void rerank_kernel(const void *db, const float *xn, int64_t dim, const void *q,
                              const float *qn, int len, int P, uint32_t *ids, float *dists) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t *s = reinterpret_cast<uint64_t *>(smem);
    __shared__ int valid;
    const int64_t j = blockIdx.x;
    uint32_t *rid = ids + j * len;
    float *rd = dists + j * len;
    if (threadIdx.x == 0) {
        int v = 0;
        while (v < len && rid[v] != 0) ++v;
        valid = v;
    }
    __syncthreads();
    const int nv = valid;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        if (i < nv) {
            const uint32_t id = rid[i];
            const float d = exact_pair<METRIC>(db, int64_t(id) - 1, dim, q, j, xn, qn);
            s[i] = make_key(d, id - 1);
        } else {
            s[i] = KEY_EMPTY;
        }
    }
    block_bitonic_sort(s, P);
    for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        rid[i] = key_id0(s[i]) + 1;
        rd[i] = key_dist(s[i]);
    }
}

}  // namespace

cudaError_t launch_rerank(int metric, const void *db, const float *db_norm, int64_t dim,
                          const void *q, const float *q_norm, int64_t m, int len,
                          uint32_t *ids, float *dists, cudaStream_t st, int *launches) {
    if (m <= 0 || len <= 0) return cudaSuccess;
    const int P = next_pow2(len);
    const size_t smem = size_t(P) * 8;
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    if (launches) *launches += 1;
#define SSG_RR(MET)                                                                               \
    case MET: {                                                                                   \
        cudaError_t e = cudaFuncSetAttribute(rerank_kernel<MET>,                                  \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)); \
        if (e != cudaSuccess) return e;                                                           \
        rerank_kernel<MET><<<unsigned(m), 128, smem, st>>>(db, db_norm, dim, q, q_norm, len, P,   \
                                                           ids, dists);                            \
        return cudaGetLastError();                                                                \
    }
    switch (metric) {
        SSG_RR(SQL2)
        SSG_RR(L2)
        SSG_RR(NORMCOSINE)
        SSG_RR(COSINE)
        SSG_RR(IP)
        SSG_RR(HAMMING)
        default: return cudaErrorInvalidValue;
    }
#undef SSG_RR
}

}  // namespace ssg
