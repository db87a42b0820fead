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

// Exact FP32 distance of the row x to the query q (both dim floats, in
// global or shared memory), summed in index order with one FMA per element;
// xn, qn are the norms Cosine divides by.
template <int METRIC>
__device__ __forceinline__ float exact_rows(const float *x, const float *q, int64_t dim, float xn, float qn) {
    float acc = 0.0f;
    int64_t c = 0;
    // 16-byte loads where both rows allow them (the same elements in the same
    // order: the sum is unchanged)
    if (((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(q)) & 15) == 0) {
        const float4 *x4 = reinterpret_cast<const float4 *>(x);
        const float4 *q4 = reinterpret_cast<const float4 *>(q);
        for (; c + 4 <= dim; c += 4) {
            const float4 a = x4[c / 4], b = q4[c / 4];
            if constexpr (METRIC == SQL2 || METRIC == L2) {
                float m = a.x - b.x; acc = fmaf(m, m, acc);
                m = a.y - b.y; acc = fmaf(m, m, acc);
                m = a.z - b.z; acc = fmaf(m, m, acc);
                m = a.w - b.w; acc = fmaf(m, m, acc);
            } else {
                acc = fmaf(a.x, b.x, acc);
                acc = fmaf(a.y, b.y, acc);
                acc = fmaf(a.z, b.z, acc);
                acc = fmaf(a.w, b.w, acc);
            }
        }
    }
    if constexpr (METRIC == SQL2 || METRIC == L2) {
        for (; c < dim; ++c) { float m = x[c] - q[c]; acc = fmaf(m, m, acc); }
        return METRIC == L2 ? sqrtf(acc) : acc;
    } else {
        for (; c < dim; ++c) acc = fmaf(x[c], q[c], acc);
        if (METRIC == NORMCOSINE) return 1.0f - acc;
        if (METRIC == IP) return -acc;
        return 1.0f - acc / (xn * qn);
    }
}

// Exact distance of one (row, query) pair, summed in index order with one FMA
// per element -- the same chain as the scan kernels and the oracle.
template <int METRIC>
__device__ __forceinline__ float exact_pair(const void *dbv, int64_t row, int64_t dim, const void *qv, int64_t j,
                            const float *xn, const float *qn) {
    if constexpr (METRIC == HAMMING) {
        const uint64_t *x = static_cast<const uint64_t *>(dbv) + row * dim;
        const uint64_t *q = static_cast<const uint64_t *>(qv) + j * dim;
        int d = 0;
        for (int64_t w = 0; w < dim; ++w) d += __popcll(x[w] ^ q[w]);
        return float(d);
    } else {
        const float *x = static_cast<const float *>(dbv) + row * dim;
        const float *q = static_cast<const float *>(qv) + j * dim;
        return exact_rows<METRIC>(x, q, dim, METRIC == COSINE ? xn[row] : 0.0f, METRIC == COSINE ? qn[j] : 0.0f);
    }
}

}  // namespace ssg
