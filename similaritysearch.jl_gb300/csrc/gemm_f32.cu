// gemm_f32.cu -- plain FP32 scan as a register-tiled SIMT contraction.
//
// The plain method's fast path.  A CTA computes a 128-query x 128-row tile
// of dot products with 8x8 accumulators per thread (FFMA, k in index order,
// so every dot product is the same fma chain as search(::ExhaustiveSearch)'s
// `d = muladd(a_i, b_i, d)`, src/dist/cos.jl:78-84).  Database and queries
// are kept in HBM as k-major tiles (per 128 rows: dim-major, 128 floats per
// dim, zero-padded), so a slice of BK dims is one contiguous 8 KB block that
// 16-byte cp.async copies land in shared memory in exactly the layout the
// inner loop reads (STAGES-deep ring, no registers spent on staging, two
// CTAs per SM).  After the last slice the tile is staged in two 64-row halves
// through the operand buffers; thread r (r < 128) owns query row r and pushes
// its 128 values into its top-k.
//   * NormCosine / InnerProduct / Cosine: the tile values ARE the exact FP32
//     distances (1 - dot, -dot, 1 - dot / (|x| |q|)), so the keys are final.
//   * SqL2 / L2: the tile holds |x|^2 - 2 x.q (the query's |q|^2 is common to
//     the row and dropped).  That GEMM form differs from the reference's
//     difference form sum (x_i - q_i)^2 (src/dist/vecs.jl:93-102) by
//     rounding, so kk = k + margin candidates are kept and re-scored exactly
//     in finalize_rerank_kernel, which checks that the margin provably covers
//     the exact top k and flags the query for the exact direct scan otherwise.
#include "common.cuh"
#include "kernels.h"

namespace ssg {

namespace {

constexpr int BM = 128;       // queries per CTA
constexpr int BN = 128;       // database rows per tile
#ifndef SSG_GEMM_BK
#define SSG_GEMM_BK 16
#endif
#ifndef SSG_GEMM_STAGES
#define SSG_GEMM_STAGES 3
#endif
constexpr int BK = SSG_GEMM_BK;  // dims per pipeline stage
constexpr int LDA = BM;       // k-major slice row (floats): the tile layout in HBM
constexpr int SROW = BN + 4;  // staged tile row stride (floats)
constexpr int THREADS = 256;
constexpr int STAGES = SSG_GEMM_STAGES;  // cp.async ring depth (STAGES - 1 slices in flight ahead)
constexpr int kBufCap = 12;       // buffered top-k: drain checked every 8 values, trigger 4
constexpr int kDrainTrigger = 4;

struct GemmSmem {
    // operand ring, also holding a staged half tile in the epilogue
    __host__ __device__ static constexpr size_t operands() {
        return size_t(STAGES) * 2 * BK * LDA * 4 > size_t(BM / 2) * SROW * 4 ? size_t(STAGES) * 2 * BK * LDA * 4
                                                                             : size_t(BM / 2) * SROW * 4;
    }
    static size_t heaps(int kk) { return size_t(BM) * (kk + kBufCap) * 8; }
    static size_t total(int kk) { return operands() + heaps(kk); }
};

template <int METRIC>
__device__ __forceinline__ float gemm_value(float acc, float xaux, float qn) {
    if (METRIC == NORMCOSINE) return 1.0f - acc;
    if (METRIC == IP) return -acc;
    if (METRIC == COSINE) return 1.0f - acc / (xaux * qn);
    return fmaf(-2.0f, acc, xaux);  // SQL2 / L2: |x|^2 - 2 x.q
}

__device__ __forceinline__ void cp_async16(float *dst, const float *src) {
    const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
// all but the STAGES - 2 most recently committed groups are complete
__device__ __forceinline__ void cp_async_wait_ahead() {
    asm volatile("cp.async.wait_group %0;" ::"n"(STAGES - 2) : "memory");
}

// Issues the copies of the k-slice [k0, k0+BK) of a k-major tile (BK * 128
// contiguous floats) into the slice buffer s: 16 bytes per thread and pass.
__device__ __forceinline__ void load_slice_async(float *s, const float *__restrict__ tile, int k0) {
    const float *src = tile + size_t(k0) * BM;
#pragma unroll
    for (int i = threadIdx.x; i < BK * BM / 4; i += THREADS) cp_async16(s + i * 4, src + i * 4);
}

// k-major tiles: out[(t * kpad + k) * 128 + r] = x[(t * 128 + r) * dim + k],
// zero for rows >= rows or k >= dim.  A block transposes 32 rows x 32 dims
// through shared memory (coalesced reads and writes).
__global__ void gemm_tile_kernel(const float *__restrict__ x, int64_t rows, int dim, int kpad, int64_t tiles,
                                 float *__restrict__ out) {
    __shared__ float t[32][33];
    const int64_t r0 = int64_t(blockIdx.x) * 32;  // row block (within all padded rows)
    const int k0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int64_t r = r0 + i;
        const int k = k0 + threadIdx.x;
        t[i][threadIdx.x] = (r < rows && k < dim) ? x[r * dim + k] : 0.0f;
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int k = k0 + i;
        const int64_t r = r0 + threadIdx.x;
        if (k < kpad && r < tiles * BM) out[((r / BM) * kpad + k) * BM + (r % BM)] = t[threadIdx.x][i];
    }
}

// acc[i][j] = sum_k A[row_i][k] * B[col_j][k] over the k-major tiles `qtile`
// (rows ty*4+i and 64+ty*4+i) and `dtile` (columns tx*4+j and 64+tx*4+j),
// one fmaf per k in increasing k: the sequential dot-product chain.  Uses
// the operand ring sA / sB; the caller has synchronised before it is reused.
__device__ __forceinline__ void tile_products(float (&acc)[8][8], float *sA, float *sB, const float *qtile,
                                              const float *dtile, int kpad) {
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int nslices = kpad / BK;
    // prologue: slices 0 .. STAGES-2 in flight (one commit group each, maybe empty)
#pragma unroll
    for (int p = 0; p < STAGES - 1; ++p) {
        if (p < nslices) {
            load_slice_async(sA + p * BK * LDA, qtile, p * BK);
            load_slice_async(sB + p * BK * LDA, dtile, p * BK);
        }
        cp_async_commit();
    }
    for (int sl = 0; sl < nslices; ++sl) {
        cp_async_wait_ahead();
        __syncthreads();  // slice sl visible; the buffer of slice sl-1 is free
        if (sl + STAGES - 1 < nslices) {
            const int nb = (sl + STAGES - 1) % STAGES;
            load_slice_async(sA + nb * BK * LDA, qtile, (sl + STAGES - 1) * BK);
            load_slice_async(sB + nb * BK * LDA, dtile, (sl + STAGES - 1) * BK);
        }
        cp_async_commit();
        const int buf = sl % STAGES;
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
    }
    cp_async_wait_all();
}

// Bit sketches: bit c of row r's sketch is set iff sum_k X[r][k] * R[c][k] >= 0
// (sequential fma chain), packed 64 coordinates per UInt64 word, coordinate c
// in bit c % 64 of word c / 64 (bitsketch / packsigns, src/proj/bitsketches.jl:
// 19-32,56-57,101-104; transform!, src/proj/Projections.jl:137-143).  A CTA
// computes a 128-row x 128-coordinate tile and writes 128 x 2 words.
__global__ void __launch_bounds__(THREADS, 2)
bitsketch_kernel(const float *__restrict__ xtiles, const float *__restrict__ rtiles, int kpad, int64_t n, int outdim,
                 int words, uint64_t *__restrict__ out) {
    extern __shared__ __align__(16) unsigned char smem[];
    float *sA = reinterpret_cast<float *>(smem);
    float *sB = sA + STAGES * BK * LDA;
    uint8_t *sbits = smem;  // [128][128] sign bytes, aliases the operands after the products
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
    tile_products(acc, sA, sB, xtiles + size_t(blockIdx.x) * kpad * BM, rtiles + size_t(blockIdx.y) * kpad * BN,
                  kpad);
    __syncthreads();  // operands no longer read
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int r = (i < 4 ? 0 : 64) + ty * 4 + (i & 3);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int c = (j < 4 ? 0 : 64) + tx * 4 + (j & 3);
            sbits[r * BN + c] = acc[i][j] >= 0.0f ? 1 : 0;
        }
    }
    __syncthreads();
    // thread -> (row, 64-coordinate half): one output word
    const int r = tid >> 1, h = tid & 1;
    const int64_t row = int64_t(blockIdx.x) * BM + r;
    const int word = blockIdx.y * 2 + h;
    if (row >= n || word >= words) return;
    uint64_t w = 0;
    const uint8_t *src = sbits + r * BN + h * 64;
    for (int b = 0; b < 64; ++b) {
        const int c = word * 64 + b;
        if (c < outdim && src[b]) w |= uint64_t(1) << b;
    }
    out[size_t(row) * words + word] = w;
}

template <int METRIC>
__global__ void __launch_bounds__(THREADS, 2)
gemm_f32_kernel(ScanArgs a, int kpad, const float *__restrict__ dtiles, const float *__restrict__ xaux,
                const float *__restrict__ qtiles, const float *__restrict__ qn) {
    extern __shared__ __align__(16) unsigned char smem[];
    float *sA = reinterpret_cast<float *>(smem);  // [STAGES][BK][LDA]
    float *sB = sA + STAGES * BK * LDA;            // [STAGES][BK][LDA]
    float *sT = sA;                                // staged half tile [64][SROW], aliases the operands
    uint64_t *heaps = reinterpret_cast<uint64_t *>(smem + GemmSmem::operands());
    uint64_t *bufs = heaps + size_t(BM) * a.kk;

    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int64_t q0 = int64_t(blockIdx.x) * BM;
    const int64_t lo = int64_t(blockIdx.y) * a.split_len;  // a multiple of BN
    const int64_t hi = lo + a.split_len < a.n ? lo + a.split_len : a.n;
    const float *qtile = qtiles + size_t(blockIdx.x) * kpad * BM;

    // thread r < 128 owns query row r (warps 0-3)
    const bool owner = tid < BM;
    const bool row_valid = owner && q0 + tid < a.m;
    BufferedTopK T;
    if (owner) T.init(heaps + tid, bufs + tid, a.kk, BM);
    // the query's bound shared with the other splits (ScanArgs::qbound)
    uint32_t *qb = (a.qbound && row_valid) ? a.qbound + q0 + tid : nullptr;
    float published = INFINITY;

    for (int64_t j0 = lo; j0 < hi; j0 += BN) {
        float acc[8][8];
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;

        __syncthreads();  // the previous tile's epilogue is done with shared memory
        tile_products(acc, sA, sB, qtile, dtiles + size_t(j0 / BN) * kpad * BN, kpad);
        // epilogue, in two halves of 64 query rows staged through the operands
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            __syncthreads();  // operands (or the previous half) no longer read
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int lr = ty * 4 + i;        // row within the half
                const int qr = h * 64 + lr;       // query row within the tile
                const float qq = (METRIC == COSINE && q0 + qr < a.m) ? qn[q0 + qr] : 1.0f;
#pragma unroll
                for (int hc = 0; hc < 2; ++hc) {
                    const int cb = hc * 64 + tx * 4;
                    float4 v;
                    float *pv = reinterpret_cast<float *>(&v);
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const int64_t id = j0 + cb + j;
                        const float aux = (METRIC == NORMCOSINE || METRIC == IP) ? 0.0f
                                          : (id < hi ? xaux[id] : 0.0f);
                        pv[j] = gemm_value<METRIC>(acc[h * 4 + i][hc * 4 + j], aux, qq);
                    }
                    *reinterpret_cast<float4 *>(sT + lr * SROW + cb) = v;
                }
            }
            __syncthreads();
            // warps 2h and 2h+1 own rows [64h, 64h + 64)
            if ((tid >> 6) == h) {
                const float *row = sT + (tid - h * 64) * SROW;
                const float bnd = qb ? bound_read(qb) : INFINITY;
                float thr = row_valid ? fminf(T.topd, bnd) : -INFINITY;
                // a group of 8 values is only looked at when one of the warp's
                // rows may take one of them (padding rows take none)
#pragma unroll 2
                for (int c = 0; c < BN; c += 8) {
                    const float4 v0 = *reinterpret_cast<const float4 *>(row + c);
                    const float4 v1 = *reinterpret_cast<const float4 *>(row + c + 4);
                    const float gm = fmin3(fmin3(v0.x, v0.y, v0.z), fmin3(v0.w, v1.x, v1.y), fminf(v1.z, v1.w));
                    if (!__any_sync(0xffffffffu, gm <= thr)) continue;
                    const float vv[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const int64_t id = j0 + c + j;
                        if (row_valid && vv[j] <= thr && id < hi) T.append(vv[j], uint32_t(id + a.id_base));
                    }
                    T.maybe_drain(kDrainTrigger);
                    if (row_valid) thr = fminf(T.topd, bnd);
                }
                if (qb && T.topd < published) {
                    bound_lower(qb, T.topd);
                    published = T.topd;
                }
            }
        }
    }
    if (owner) {
        T.drain();
        if (row_valid) {
            T.H.sort_ascending();
            uint64_t *out = a.cand + (size_t(q0 + tid) * a.splits + blockIdx.y) * a.kk;
            for (int i = 0; i < a.kk; ++i) out[i] = T.H.h[i * BM];
        }
    }
}

template <int METRIC>
cudaError_t launch_gemm_t(const ScanArgs &a, int kpad, const float *dtiles, const float *xaux, const float *qtiles,
                          const float *qn, cudaStream_t st) {
    const size_t smem = GemmSmem::total(a.kk);
    auto kern = gemm_f32_kernel<METRIC>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    dim3 grid(unsigned((a.m + BM - 1) / BM), unsigned(a.splits));
    kern<<<grid, THREADS, smem, st>>>(a, kpad, dtiles, xaux, qtiles, qn);
    return cudaGetLastError();
}

}  // namespace

bool gemm_fits(int kk) { return GemmSmem::total(kk) <= size_t(220) * 1024; }

// resident CTAs per SM (the kernel is bounded to 2; shared memory may allow 1)
int gemm_ctas_per_sm(int kk) { return GemmSmem::total(kk) + 1024 <= size_t(114) * 1024 ? 2 : 1; }

int gemm_kpad(int64_t dim) { return int((dim + BK - 1) / BK * BK); }
size_t gemm_tile_floats(int64_t dim) { return size_t(gemm_kpad(dim)) * BM; }

cudaError_t launch_gemm_tiles(const float *x, int64_t rows, int64_t dim, int64_t tiles, float *out, cudaStream_t st,
                              int *launches) {
    if (tiles <= 0) return cudaSuccess;
    const int kpad = gemm_kpad(dim);
    dim3 grid(unsigned(tiles * BM / 32), unsigned((kpad + 31) / 32));
    if (launches) *launches += 1;
    gemm_tile_kernel<<<grid, dim3(32, 8), 0, st>>>(x, rows, int(dim), kpad, tiles, out);
    return cudaGetLastError();
}

cudaError_t launch_bitsketch(const float *xtiles, const float *rtiles, int64_t dim, int64_t n, int64_t outdim,
                             uint64_t *out, cudaStream_t st, int *launches) {
    if (n <= 0 || outdim <= 0) return cudaSuccess;
    const int kpad = gemm_kpad(dim);
    const int words = int((outdim + 63) / 64);
    const size_t smem = GemmSmem::operands() > size_t(BM) * BN ? GemmSmem::operands() : size_t(BM) * BN;
    cudaError_t e = cudaFuncSetAttribute(bitsketch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    dim3 grid(unsigned((n + BM - 1) / BM), unsigned((outdim + BN - 1) / BN));
    if (launches) *launches += 1;
    bitsketch_kernel<<<grid, THREADS, smem, st>>>(xtiles, rtiles, kpad, n, int(outdim), words, out);
    return cudaGetLastError();
}

cudaError_t launch_gemm_f32(const ScanArgs &a, const float *dtiles, const float *xaux, const float *qtiles,
                            const float *q_norm, cudaStream_t st, int *launches) {
    if (!gemm_fits(a.kk) || a.split_len % BN) return cudaErrorInvalidValue;
    const int kpad = gemm_kpad(a.dim);
    if (launches) *launches += 1;
    switch (a.metric) {
        case SQL2: return launch_gemm_t<SQL2>(a, kpad, dtiles, xaux, qtiles, q_norm, st);
        case L2: return launch_gemm_t<L2>(a, kpad, dtiles, xaux, qtiles, q_norm, st);
        case NORMCOSINE: return launch_gemm_t<NORMCOSINE>(a, kpad, dtiles, xaux, qtiles, q_norm, st);
        case COSINE: return launch_gemm_t<COSINE>(a, kpad, dtiles, xaux, qtiles, q_norm, st);
        case IP: return launch_gemm_t<IP>(a, kpad, dtiles, xaux, qtiles, q_norm, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace ssg
