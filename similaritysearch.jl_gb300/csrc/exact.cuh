// exact.cuh -- the exact FP32 distance of one (database row, query) pair.
//
// Summed in index order with one FMA per element (SqL2: m = x_i - q_i,
// d = fma(m, m, d), src/dist/vecs.jl:93-102; dot products: d = fma(x_i, q_i, d),
// src/dist/cos.jl:78-84), which is the chain the scan kernels and the oracle
// use, so every path reports bit-identical distances.
#pragma once
#include <cstdint>
#include "kernels.h"

namespace ssg {

// Exact distance of one (row, query) pair, summed in index order with one FMA
// per element -- the same chain as the scan kernels and the oracle.
template <int METRIC>
__device__ __forceinline__ float exact_pair(const void *dbv, int64_t row, int64_t dim, const void *qv, int64_t j,
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
    if constexpr (METRIC == SQL2 || METRIC == L2) {
        for (int64_t c = 0; c < dim; ++c) { float m = x[c] - q[c]; acc = fmaf(m, m, acc); }
        return METRIC == L2 ? sqrtf(acc) : acc;
    } else {
        for (int64_t c = 0; c < dim; ++c) acc = fmaf(x[c], q[c], acc);
        if (METRIC == NORMCOSINE) return 1.0f - acc;
        if (METRIC == IP) return -acc;
        return 1.0f - acc / (xn[row] * qn[j]);
    }
}

}  // namespace ssg
