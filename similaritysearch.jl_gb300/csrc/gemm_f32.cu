// gemm_f32.cu -- plain FP32 scan as a register-tiled SIMT contraction.
//
// The plain method's fast path.  A CTA computes a 128-query x 128-row tile
// of dot products with 8x8 accumulators per thread (FFMA, k in index order,
// so every dot product is the same fma chain as search(::ExhaustiveSearch)'s
// `d = muladd(a_i, b_i, d)`, src/dist/cos.jl:78-84), stages the tile in
// shared memory and lets each thread push half a row into its private top-k
// heap.
//   * NormCosine / InnerProduct / Cosine: the tile values ARE the exact FP32
//     distances (1 - dot, -dot, 1 - dot / (|x| |q|)), so the keys are final.
//   * SqL2 / L2: the tile holds |x|^2 - 2 x.q (the query's |q|^2 is common to
//     the row and dropped).  That GEMM form differs from the reference's
//     difference form sum (x_i - q_i)^2 (src/dist/vecs.jl:93-102) by
//     rounding, so kk = k + margin candidates are kept and re-scored exactly
//     in finalize_rerank_kernel, which also checks that the margin provably
//     covers the exact top k (see rerank_check below) and flags the query
//     for the exact direct scan otherwise.
#include "common.cuh"
#include "kernels.h"

namespace ssg {

namespace {

constexpr int BM = 128;       // queries per CTA
constexpr int BN = 128;       // database rows per tile
constexpr int BK = 16;        // dims per pipeline stage
constexpr int PAD = 4;        // smem row padding (floats)
constexpr int LDA = BM + PAD;
constexpr int SROW = BN + PAD;  // staged tile row stride
constexpr int THREADS = 256;

struct GemmSmem {
    static size_t operands() { return size_t(2) * BK * (LDA + LDA) * 4; }
    static size_t stage() { return size_t(BM) * SROW * 4; }
    static size_t heaps(int kk) { return size_t(THREADS) * kk * 8; }
    static size_t total(int kk) { return operands() + stage() + heaps(kk); }
};

template <int METRIC>
__device__ __forceinline__ float gemm_value(float acc, float xaux, float qn) {
    if (METRIC == NORMCOSINE) return 1.0f - acc;
    if (METRIC == IP) return -acc;
    if (METRIC == COSINE) return 1.0f - acc / (xaux * qn);
    return fmaf(-2.0f, acc, xaux);  // SQL2 / L2: |x|^2 - 2 x.q
}

// Loads the BK-wide k-slice [k0, k0+BK) of 128 rows (rows >= rows_valid or
// columns >= dim read as 0) into registers: thread -> (row = tid/2, 8 dims).
__device__ __forceinline__ void load_slice(const float *__restrict__ base, int64_t row0, int64_t rows_valid,
                                           int dim, int k0, float (&r)[8]) {
    const int tid = threadIdx.x;
    const int row = tid >> 1;
    const int c0 = (tid & 1) * 8;
    const int64_t gr = row0 + row;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int c = k0 + c0 + i;
        r[i] = (gr < rows_valid && c < dim) ? base[gr * dim + c] : 0.0f;
    }
}

__device__ __forceinline__ void store_slice(float *__restrict__ s, const float (&r)[8]) {
    const int tid = threadIdx.x;
    const int row = tid >> 1;
    const int c0 = (tid & 1) * 8;
#pragma unroll
    for (int i = 0; i < 8; ++i) s[(c0 + i) * LDA + row] = r[i];
}

template <int METRIC>
__global__ void __launch_bounds__(THREADS, 1)
gemm_f32_kernel(ScanArgs a, const float *__restrict__ db, const float *__restrict__ xaux,
                const float *__restrict__ Q, const float *__restrict__ qn) {
    extern __shared__ __align__(16) unsigned char smem[];
    float *sA = reinterpret_cast<float *>(smem);            // [2][BK][LDA]
    float *sB = sA + 2 * BK * LDA;                           // [2][BK][LDA]
    float *sT = sB + 2 * BK * LDA;                           // [BM][SROW]
    uint64_t *heaps = reinterpret_cast<uint64_t *>(sT + BM * SROW);

    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int64_t q0 = int64_t(blockIdx.x) * BM;
    const int64_t lo = int64_t(blockIdx.y) * a.split_len;
    const int64_t hi = lo + a.split_len < a.n ? lo + a.split_len : a.n;
    const int dim = int(a.dim);

    // heap owner: query row hq, columns [hh*64, hh*64+64)
    const int hq = tid >> 1, hh = tid & 1;
    Heap H{heaps + tid, a.kk, THREADS};
    H.init();
    uint64_t top = KEY_EMPTY;
    float topd = INFINITY;
    const bool hq_valid = q0 + hq < a.m;
    const float hqn = (METRIC == COSINE && hq_valid) ? qn[q0 + hq] : 1.0f;

    for (int64_t j0 = lo; j0 < hi; j0 += BN) {
        float acc[8][8];
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;

        float ra[8], rb[8];
        load_slice(Q, q0, a.m, dim, 0, ra);
        load_slice(db, j0, hi, dim, 0, rb);
        __syncthreads();  // the previous tile's epilogue is done with shared memory
        store_slice(sA, ra);
        store_slice(sB, rb);
        __syncthreads();
        int buf = 0;
        for (int k0 = 0; k0 < dim; k0 += BK) {
            const bool more = k0 + BK < dim;
            if (more) {
                load_slice(Q, q0, a.m, dim, k0 + BK, ra);
                load_slice(db, j0, hi, dim, k0 + BK, rb);
            }
            const float *cA = sA + buf * BK * LDA;
            const float *cB = sB + buf * BK * LDA;
#pragma unroll
            for (int kk = 0; kk < BK; ++kk) {
                const float4 a0 = *reinterpret_cast<const float4 *>(cA + kk * LDA + ty * 4);
                const float4 a1 = *reinterpret_cast<const float4 *>(cA + kk * LDA + 64 + ty * 4);
                const float4 b0 = *reinterpret_cast<const float4 *>(cB + kk * LDA + tx * 4);
                const float4 b1 = *reinterpret_cast<const float4 *>(cB + kk * LDA + 64 + tx * 4);
                const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(bv[j], av[i], acc[i][j]);
            }
            if (more) {
                store_slice(sA + (buf ^ 1) * BK * LDA, ra);
                store_slice(sB + (buf ^ 1) * BK * LDA, rb);
            }
            __syncthreads();
            buf ^= 1;
        }
        // stage the tile: row = query, column = database row
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int qr = (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int cb = h * 64 + tx * 4;
                float4 v;
                float *pv = reinterpret_cast<float *>(&v);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int64_t id = j0 + cb + j;
                    const float aux = (METRIC == NORMCOSINE || METRIC == IP) ? 0.0f
                                      : (id < hi ? xaux[id] : 0.0f);
                    const float qq = (METRIC == COSINE && q0 + qr < a.m) ? qn[q0 + qr] : 1.0f;
                    pv[j] = gemm_value<METRIC>(acc[i][h * 4 + j], aux, qq);
                }
                *reinterpret_cast<float4 *>(sT + qr * SROW + cb) = v;
            }
        }
        __syncthreads();
        if (hq_valid) {
            const float *row = sT + hq * SROW + hh * 64;
            const int64_t idb = j0 + hh * 64;
#pragma unroll 4
            for (int c = 0; c < 64; c += 4) {
                const float4 v = *reinterpret_cast<const float4 *>(row + c);
                const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int64_t id = idb + c + j;
                    if (vv[j] <= topd && id < hi) {
                        const uint64_t key = make_key(vv[j], uint32_t(id + a.id_base));
                        if (key < top) {
                            top = H.replace_top(key);
                            topd = (top == KEY_EMPTY) ? INFINITY : key_dist(top);
                        }
                    }
                }
            }
        }
        (void)hqn;
    }
    if (hq_valid) {
        H.sort_ascending();
        // segments per query: splits x 2 halves
        uint64_t *out = a.cand + ((size_t(q0 + hq) * a.splits + blockIdx.y) * 2 + hh) * a.kk;
        for (int i = 0; i < a.kk; ++i) out[i] = H.h[i * THREADS];
    }
}

template <int METRIC>
cudaError_t launch_gemm_t(const ScanArgs &a, const float *db, const float *xaux, const float *q, const float *qn,
                          cudaStream_t st) {
    const size_t smem = GemmSmem::total(a.kk);
    auto kern = gemm_f32_kernel<METRIC>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    dim3 grid(unsigned((a.m + BM - 1) / BM), unsigned(a.splits));
    kern<<<grid, THREADS, smem, st>>>(a, db, xaux, q, qn);
    return cudaGetLastError();
}

}  // namespace

bool gemm_fits(int kk) { return GemmSmem::total(kk) <= size_t(220) * 1024; }

cudaError_t launch_gemm_f32(const ScanArgs &a, const float *db, const float *xaux, const float *q,
                            const float *q_norm, cudaStream_t st, int *launches) {
    if (!gemm_fits(a.kk)) return cudaErrorInvalidValue;
    if (launches) *launches += 1;
    switch (a.metric) {
        case SQL2: return launch_gemm_t<SQL2>(a, db, xaux, q, q_norm, st);
        case L2: return launch_gemm_t<L2>(a, db, xaux, q, q_norm, st);
        case NORMCOSINE: return launch_gemm_t<NORMCOSINE>(a, db, xaux, q, q_norm, st);
        case COSINE: return launch_gemm_t<COSINE>(a, db, xaux, q, q_norm, st);
        case IP: return launch_gemm_t<IP>(a, db, xaux, q, q_norm, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace ssg
