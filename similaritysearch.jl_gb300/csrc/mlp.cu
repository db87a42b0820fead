// mlp.cu -- kernels of the learned shortlist: a small MLP (d -> H (ReLU) -> E)
// trained with a triplet loss, forward and backward written by hand.
//
// Every product of the network -- forward, both weight gradients and the
// hidden-layer gradient -- runs on the 5th-generation tensor cores
// (tcgen05.mma kind::f16: BF16 operands, FP32 accumulators in TMEM), in one
// GEMM kernel that covers all of their operand layouts.  Its threads stage
// the FP32 operands into shared memory as BF16 tiles in the tensor core's
// swizzled K-major layout (128-byte rows, 128-byte swizzle), reading rows
// K-contiguously or, for a transposed operand, M-contiguously (coalesced
// either way), while one thread issues the MMAs of the previous K-block: two
// stages, an mbarrier per stage signalled by tcgen05.commit.  The epilogue
// reads the accumulator with tcgen05.ld, turns each 32 x 32 block through
// shared memory (coalesced row writes) and applies what the caller fused
// in: bias, ReLU, a ReLU-derivative mask, and per-tile column sums (the bias
// gradients, reduced in a fixed order later, so training is deterministic).
// The products are small, so each is split along K over enough CTAs that
// every CTA walks about two K-blocks; each split writes its own partial
// product, summed in a fixed order by a reduction kernel that applies the
// bias and ReLU (forward products) or by Adam (weight gradients).
//
// `exact` mode: each operand element x is split into three BF16 pieces,
// hi = bf16(x), mid = bf16(x - hi), lo = bf16(x - hi - mid) (24 significant
// bits, as many as FP32 holds), and six MMAs accumulate every piece product
// of weight 2^-16 or more: hi.hi + hi.mid + mid.hi + hi.lo + mid.mid + lo.hi
// (the dropped ones are below 2^-24 relative).  The gradient check runs the
// same kernels in this mode against an FP64 oracle, at FP32-class accuracy;
// training and embedding use plain BF16 operands.
#include "kernels.h"
#include "tc_ptx.cuh"

#include <cuda_bf16.h>

namespace ssg {

namespace {

constexpr int BM = 128;          // rows per tile (TMEM lanes)
constexpr int BK = 64;           // K elements per K-block: one 128-byte BF16 row
constexpr int SWB = 128;         // swizzle bytes
constexpr int GT = 128;          // threads per CTA (4 warps: one TMEM lane quarter each)

template <int BN, bool EXACT>
struct GemmSmem {
    static constexpr int a_bytes = BM * SWB;             // 16 KB
    static constexpr int b_bytes = BN * SWB;
    static constexpr int stage = (a_bytes + b_bytes) * (EXACT ? 3 : 1);  // hi (, mid, lo)
    static constexpr int total = 1024 + 2 * stage + 4 * BN * 4 + 64;
};

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Stages rows [r0, r0 + R) x K-block [k0, k0 + BK) of an FP32 operand into a
// BF16 tile (hi) and, in exact mode, the tiles of its second and third
// pieces (mid, lo) at `piece` bytes after it.  kmajor: element (r, k) at
// X[r * ld + k], else at X[k * ld + r].  Out-of-range elements are 0.
// Two phases: every load of the thread's chunks is issued first (registers),
// then they are converted and stored, so a K-block costs about one global
// load latency instead of one per chunk.
template <int R>
struct Staged {
    static constexpr int CPT = R * (BK / 8) / GT;  // 16-byte chunks per thread
    float v[CPT][8];
};

template <int R>
__device__ __forceinline__ void load_operand(Staged<R> &t, const float *__restrict__ X, int64_t ld, int kmajor, int r0,
                                             int rlim, int k0, int klim, bool vec4) {
#pragma unroll
    for (int i = 0; i < Staged<R>::CPT; ++i) {
        const int c = int(threadIdx.x) + i * GT;
        int r, kc;
        if (kmajor) { r = c / (BK / 8); kc = c % (BK / 8); }
        else { kc = c / R; r = c % R; }  // consecutive threads: consecutive rows (coalesced)
        const int gr = r0 + r, gk = k0 + kc * 8;
        float *v = t.v[i];
        if (gr < rlim && kmajor && vec4 && gk + 8 <= klim) {
            const float *p = X + int64_t(gr) * ld + gk;
            const float4 a = __ldg(reinterpret_cast<const float4 *>(p));
            const float4 b = __ldg(reinterpret_cast<const float4 *>(p + 4));
            v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
        } else if (gr < rlim && kmajor) {
            const float *p = X + int64_t(gr) * ld + gk;
#pragma unroll
            for (int j = 0; j < 8; ++j) v[j] = gk + j < klim ? __ldg(p + j) : 0.0f;
        } else if (gr < rlim) {
#pragma unroll
            for (int j = 0; j < 8; ++j) v[j] = gk + j < klim ? __ldg(X + int64_t(gk + j) * ld + gr) : 0.0f;
        } else {
#pragma unroll
            for (int j = 0; j < 8; ++j) v[j] = 0.0f;
        }
    }
}

template <int R, bool EXACT>
__device__ __forceinline__ void store_operand(const Staged<R> &t, int kmajor, uint8_t *hi, int piece) {
#pragma unroll
    for (int i = 0; i < Staged<R>::CPT; ++i) {
        const int c = int(threadIdx.x) + i * GT;
        int r, kc;
        if (kmajor) { r = c / (BK / 8); kc = c % (BK / 8); }
        else { kc = c / R; r = c % R; }
        const float *v = t.v[i];
        __align__(16) __nv_bfloat16 h[8];
        __align__(16) __nv_bfloat16 md[8];
        __align__(16) __nv_bfloat16 l[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            h[j] = __float2bfloat16_rn(v[j]);
            if (EXACT) {
                const float r1 = v[j] - __bfloat162float(h[j]);  // exact in FP32
                md[j] = __float2bfloat16_rn(r1);
                l[j] = __float2bfloat16_rn(r1 - __bfloat162float(md[j]));
            }
        }
        const uint32_t off = tc::swizzled_offset(uint32_t(r), uint32_t(kc * 16), SWB);
        *reinterpret_cast<uint4 *>(hi + off) = *reinterpret_cast<const uint4 *>(h);
        if (EXACT) {
            *reinterpret_cast<uint4 *>(hi + piece + off) = *reinterpret_cast<const uint4 *>(md);
            *reinterpret_cast<uint4 *>(hi + 2 * piece + off) = *reinterpret_cast<const uint4 *>(l);
        }
    }
}

template <int BN, bool EXACT>
__global__ void __launch_bounds__(GT, 1) mlp_gemm_kernel(MlpGemm g, int vec_a, int vec_b) {
    using S = GemmSmem<BN, EXACT>;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    float *red = reinterpret_cast<float *>(smem + 2 * S::stage);   // [4][BN] column-sum scratch
    uint64_t *bar = reinterpret_cast<uint64_t *>(red + 4 * BN);    // one per stage
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar + 2);
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int kps = (g.K + int(gridDim.z) - 1) / int(gridDim.z);
    const int kbeg = int(blockIdx.z) * ((kps + BK - 1) / BK * BK);
    const int kend = min(g.K, kbeg + (kps + BK - 1) / BK * BK);
    const int nkb = kend > kbeg ? (kend - kbeg + BK - 1) / BK : 0;

    if (threadIdx.x == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
        tc::fence_mbarrier_init();
    }
    if (warp == 0) tc::tmem_alloc<BN>(tmem_slot);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    constexpr uint32_t idesc = tc::idesc_bf16_f32(BM, BN);

    bool ok = true;
    for (int kb = 0; kb < nkb && ok; ++kb) {
        const int s = kb & 1;
        // stage: A hi, mid, lo tiles, then B hi, mid, lo tiles
        uint8_t *st = smem + s * S::stage;
        uint8_t *a_hi = st, *b_hi = st + (EXACT ? 3 : 1) * S::a_bytes;
        // the MMAs of K-block kb - 2 read this stage: wait (bounded) until
        // they are done; the CTA leaves the loop together if a wait gave up
        int waited = 1;
        if (kb >= 2) waited = tc::mbar_wait(&bar[s], ((kb - 2) >> 1) & 1, g.err, 11) ? 1 : 0;
        if (!__syncthreads_and(waited)) { ok = false; break; }
        const int k0 = kbeg + kb * BK;
        {
            Staged<BM> ta;
            Staged<BN> tb;
            load_operand<BM>(ta, g.A, g.lda, g.a_kmajor, m0, g.M, k0, kend, vec_a != 0);
            load_operand<BN>(tb, g.B, g.ldb, g.b_kmajor, n0, g.N, k0, kend, vec_b != 0);
            store_operand<BM, EXACT>(ta, g.a_kmajor, a_hi, S::a_bytes);
            store_operand<BN, EXACT>(tb, g.b_kmajor, b_hi, S::b_bytes);
        }
        fence_proxy_async();  // generic-proxy stores -> visible to the tensor core
        __syncthreads();
        if (threadIdx.x == 0) {
            tc::tc_fence_after();
            const uint32_t ah = tc::smem_u32(a_hi), bh = tc::smem_u32(b_hi);
#pragma unroll
            for (int j = 0; j < BK / 16; ++j) {
                const uint32_t o = uint32_t(j * 32);
                tc::mma_f16(tmem, tc::smem_desc(ah + o, SWB), tc::smem_desc(bh + o, SWB), idesc,
                            (kb > 0 || j > 0) ? 1u : 0u);
                if (EXACT) {
                    // (piece of A, piece of B): 0 = hi, 1 = mid, 2 = lo
                    constexpr int pa[5] = {0, 1, 0, 1, 2}, pb[5] = {1, 0, 2, 1, 0};
#pragma unroll
                    for (int t = 0; t < 5; ++t)
                        tc::mma_f16(tmem, tc::smem_desc(ah + uint32_t(pa[t] * S::a_bytes) + o, SWB),
                                    tc::smem_desc(bh + uint32_t(pb[t] * S::b_bytes) + o, SWB), idesc, 1u);
                }
            }
            tc::mma_commit(&bar[s]);
        }
    }
    // the last commit (bounded wait) before the accumulator is read or freed;
    // after a failed wait the earlier commits are waited for too
    if (nkb > 0) {
        const int last = nkb - 1;
        if (!tc::mbar_wait(&bar[last & 1], (last >> 1) & 1, g.err, 12)) ok = false;
        if (nkb > 1) tc::mbar_wait(&bar[(last - 1) & 1], ((last - 1) >> 1) & 1, g.err, 12);
    }
    ok = __syncthreads_and(ok ? 1 : 0) != 0;  // CTA-uniform: the TMEM loads below are .sync.aligned
    tc::tc_fence_after();
    // Each warp's 32 x 32 blocks pass through shared memory (the operand
    // stages are free once the last commit has arrived) so that a lane
    // writes one column and a store instruction covers 32 consecutive
    // columns of one row; the bias, ReLU, mask and column sums are applied in
    // that pass, where each lane owns one column.
    float *tile = reinterpret_cast<float *>(smem) + warp * (32 * 33);
    float *C = g.C + size_t(blockIdx.z) * size_t(g.M) * size_t(g.ldc);
    for (int c = 0; c < BN / 32; ++c) {
        float v[32];
        if (nkb > 0 && ok) {
            __syncwarp();
            tc::tmem_ld_32x32b_x32(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c * 32), v);
        } else {
#pragma unroll
            for (int j = 0; j < 32; ++j) v[j] = 0.0f;
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) tile[lane * 33 + j] = v[j];  // row = lane
        __syncwarp();
        const int n = n0 + c * 32 + lane;
        const bool nvalid = n < g.N;
        const float b = (g.bias && nvalid) ? g.bias[n] : 0.0f;
        // the mask values first (independent loads in flight together)
        float mk[32];
#pragma unroll
        for (int r = 0; r < 32; ++r) {
            const int row = m0 + warp * 32 + r;
            mk[r] = (g.mask && nvalid && row < g.M) ? __ldg(g.mask + int64_t(row) * g.ldc + n) : 1.0f;
        }
        float csum = 0.0f;
#pragma unroll
        for (int r = 0; r < 32; ++r) {
            const int row = m0 + warp * 32 + r;
            const bool valid = nvalid && row < g.M;
            float x = tile[r * 33 + lane] + b;
            if (g.relu) x = fmaxf(x, 0.0f);
            if (!(mk[r] > 0.0f)) x = 0.0f;
            if (valid) {
                C[int64_t(row) * g.ldc + n] = x;
                csum += x;
            }
        }
        if (g.colsum) red[warp * BN + c * 32 + lane] = csum;
        __syncwarp();
    }
    if (g.colsum) {
        __syncthreads();
        for (int t = threadIdx.x; t < BN; t += GT)
            if (n0 + t < g.N)
                g.colsum[int64_t(blockIdx.x) * g.N + n0 + t] = ((red[t] + red[BN + t]) + red[2 * BN + t]) + red[3 * BN + t];
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::tc_fence_after();
        tc::tmem_dealloc<BN>(tmem);
    }
}

template <int BN, bool EXACT>
cudaError_t launch_gemm_t(const MlpGemm &g, int vec_a, int vec_b, cudaStream_t st) {
    const size_t smem = GemmSmem<BN, EXACT>::total;
    auto kern = mlp_gemm_kernel<BN, EXACT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    dim3 grid(unsigned((g.M + BM - 1) / BM), unsigned((g.N + BN - 1) / BN), unsigned(g.splits));
    kern<<<grid, GT, smem, st>>>(g, vec_a, vec_b);
    return cudaGetLastError();
}

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// Triplet loss on Z = [anchors; positives; negatives] (3B rows of E):
// l = max(0, |a-p|^2 - |a-n|^2 + margin), mean over the batch; writes dL/dZ.
// One warp per triplet, lanes over the embedding's coordinates.
__global__ void triplet_kernel(const float *__restrict__ Z, int B, int E, float margin, float *__restrict__ dZ,
                               float *__restrict__ loss_sum, int *__restrict__ active) {
    const int b = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32);
    const int lane = threadIdx.x % 32;
    if (b >= B) return;
    const float *za = Z + size_t(b) * E;
    const float *zp = Z + size_t(B + b) * E;
    const float *zn = Z + size_t(2 * B + b) * E;
    float dp = 0.0f, dn = 0.0f;
    for (int e = lane; e < E; e += 32) {
        const float u = za[e] - zp[e], w = za[e] - zn[e];
        dp = fmaf(u, u, dp);
        dn = fmaf(w, w, dn);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dp += __shfl_xor_sync(0xffffffffu, dp, o);
        dn += __shfl_xor_sync(0xffffffffu, dn, o);
    }
    const float l = dp - dn + margin;
    float *ga = dZ + size_t(b) * E;
    float *gp = dZ + size_t(B + b) * E;
    float *gn = dZ + size_t(2 * B + b) * E;
    const float s = 2.0f / float(B);
    const bool act = l > 0.0f;
    if (act && lane == 0) {
        atomicAdd(loss_sum, l / float(B));
        atomicAdd(active, 1);
    }
    for (int e = lane; e < E; e += 32) {
        ga[e] = act ? s * (zn[e] - zp[e]) : 0.0f;
        gp[e] = act ? -s * (za[e] - zp[e]) : 0.0f;
        gn[e] = act ? s * (za[e] - zn[e]) : 0.0f;
    }
}

// C[m][n] = sum over p of P[p][m][n] (in order) + bias[n], ReLU: the
// epilogue of the split-K forward products.  Block = 32 columns x 8 rows,
// each thread four rows 8 apart.
__global__ void reduce_parts_kernel(const float *__restrict__ P, int parts, int M, int N, const float *__restrict__ bias,
                                    int relu, float *__restrict__ C) {
    const int n = blockIdx.y * 32 + threadIdx.x;
    if (n >= N) return;
    const int64_t stride = int64_t(M) * N;
    const float b = bias ? bias[n] : 0.0f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = blockIdx.x * 32 + i * 8 + int(threadIdx.y);
        if (r >= M) break;
        const float *src = P + int64_t(r) * N + n;
        float v = 0.0f;
#pragma unroll 4
        for (int p = 0; p < parts; ++p) v += src[p * stride];
        v += b;
        if (relu) v = fmaxf(v, 0.0f);
        C[int64_t(r) * N + n] = v;
    }
}

// Column sums of G (rows x N) in `parts` row ranges: out[p * N + n].  Block
// (32 columns x 8 row lanes); the 8 lanes are combined in a fixed order.
__global__ void colsum_parts_kernel(const float *__restrict__ G, int rows, int N, int parts, float *__restrict__ out) {
    __shared__ float s[8][33];
    const int n = blockIdx.x * 32 + threadIdx.x;
    const int p = blockIdx.y;
    const int per = (rows + parts - 1) / parts;
    const int r0 = p * per, r1 = min(rows, r0 + per);
    float acc = 0.0f;
    if (n < N)
        for (int r = r0 + int(threadIdx.y); r < r1; r += 8) acc += G[int64_t(r) * N + n];
    s[threadIdx.y][threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.y == 0 && n < N) {
        float t = 0.0f;
        for (int y = 0; y < 8; ++y) t += s[y][threadIdx.x];
        out[int64_t(p) * N + n] = t;
    }
}

// out[i] = sum over p of G[p * count + i] (parts summed in order)
__global__ void sum_parts_kernel(const float *__restrict__ G, int parts, int64_t count, float *__restrict__ out) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x) {
        float g = 0.0f;
        for (int p = 0; p < parts; ++p) g += G[int64_t(p) * count + i];
        out[i] = g;
    }
}

// X rows [part * bb, part * bb + bb) = S rows idx[part * T + off + i]: the
// anchors, positives and negatives of one batch in one launch, one block per
// row (16-byte copies when the rows allow them).
__global__ void gather3_kernel(const float *__restrict__ S, const int64_t *__restrict__ idx, int64_t T, int64_t off,
                               int bb, int d, float *__restrict__ X) {
    const int part = blockIdx.y;
    const int i = blockIdx.x;
    const float *src = S + idx[part * T + off + i] * d;
    float *dst = X + (int64_t(part) * bb + i) * d;
    if ((d & 3) == 0) {
        const float4 *s4 = reinterpret_cast<const float4 *>(src);
        float4 *d4 = reinterpret_cast<float4 *>(dst);
        for (int c = threadIdx.x; c < d / 4; c += blockDim.x) d4[c] = __ldg(s4 + c);
    } else {
        for (int c = threadIdx.x; c < d; c += blockDim.x) dst[c] = __ldg(src + c);
    }
}

// Adam on up to four parameter groups in one launch (blockIdx.y = group);
// each gradient is the sum of its `parts` partials, taken in order.
struct AdamGroups {
    float *W[4];
    const float *G[4];
    float *M[4], *V[4];
    int64_t count[4];
    int parts[4];
};

__global__ void adam_groups_kernel(AdamGroups a, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int g = blockIdx.y;
    float *__restrict__ W = a.W[g];
    const float *__restrict__ G = a.G[g];
    float *__restrict__ Mo = a.M[g];
    float *__restrict__ Vo = a.V[g];
    const int64_t count = a.count[g];
    const int parts = a.parts[g];
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x) {
        float gr = 0.0f;
        for (int p = 0; p < parts; ++p) gr += G[int64_t(p) * count + i];
        const float m = b1 * Mo[i] + (1.0f - b1) * gr;
        const float v = b2 * Vo[i] + (1.0f - b2) * gr * gr;
        Mo[i] = m;
        Vo[i] = v;
        W[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
    }
}

}  // namespace

int mlp_gemm_mtiles(int M) { return (M + BM - 1) / BM; }
int mlp_gemm_ntiles(int N) { return N <= 64 ? 1 : (N + 127) / 128; }

int mlp_splits(int K, int ctas, int want) {
    const int kblocks = (K + BK - 1) / BK;
    int s = (want + ctas - 1) / ctas;
    s = s < 1 ? 1 : s;
    s = s > kblocks ? kblocks : s;
    const int per = (kblocks + s - 1) / s;  // K-blocks per split, then as few splits as that needs
    return (kblocks + per - 1) / per;
}

cudaError_t mlp_reduce_parts(const float *P, int parts, int M, int N, const float *bias, int relu, float *C,
                             cudaStream_t st, int *launches) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    if (launches) *launches += 1;
    reduce_parts_kernel<<<dim3(unsigned((M + 31) / 32), unsigned((N + 31) / 32)), dim3(32, 8), 0, st>>>(
        P, parts, M, N, bias, relu, C);
    return cudaGetLastError();
}

cudaError_t mlp_gemm(const MlpGemm &g, cudaStream_t st, int *launches) {
    if (g.M <= 0 || g.N <= 0) return cudaSuccess;
    // split-K parts are summed later: no epilogue that is not linear in them
    if (g.splits < 1 || !g.err || (g.splits > 1 && (g.bias || g.relu || g.mask || g.colsum)))
        return cudaErrorInvalidValue;
    // 16-byte loads of K-major rows when every row start is 16-byte aligned
    const int vec_a = g.a_kmajor && g.lda % 4 == 0 && aligned16(g.A);
    const int vec_b = g.b_kmajor && g.ldb % 4 == 0 && aligned16(g.B);
    if (launches) *launches += 1;
    if (g.N <= 64) return g.exact ? launch_gemm_t<64, true>(g, vec_a, vec_b, st) : launch_gemm_t<64, false>(g, vec_a, vec_b, st);
    return g.exact ? launch_gemm_t<128, true>(g, vec_a, vec_b, st) : launch_gemm_t<128, false>(g, vec_a, vec_b, st);
}

cudaError_t mlp_triplet(const float *Z, int B, int E, float margin, float *dZ, float *loss_sum, int *active,
                        cudaStream_t st, int *launches) {
    if (launches) *launches += 1;
    triplet_kernel<<<unsigned((B + 7) / 8), 256, 0, st>>>(Z, B, E, margin, dZ, loss_sum, active);
    return cudaGetLastError();
}

cudaError_t mlp_colsum_parts(const float *G, int rows, int N, int parts, float *out, cudaStream_t st, int *launches) {
    if (launches) *launches += 1;
    colsum_parts_kernel<<<dim3(unsigned((N + 31) / 32), unsigned(parts)), dim3(32, 8), 0, st>>>(G, rows, N, parts, out);
    return cudaGetLastError();
}

cudaError_t mlp_sum_parts(const float *G, int parts, int64_t count, float *out, cudaStream_t st, int *launches) {
    if (launches) *launches += 1;
    int64_t blocks = (count + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    sum_parts_kernel<<<unsigned(blocks), 256, 0, st>>>(G, parts, count, out);
    return cudaGetLastError();
}

cudaError_t mlp_gather3(const float *S, const int64_t *idx, int64_t T, int64_t off, int bb, int d, float *X,
                        cudaStream_t st, int *launches) {
    if (bb <= 0) return cudaSuccess;
    if (launches) *launches += 1;
    const int threads = d >= 512 ? 192 : 64;
    gather3_kernel<<<dim3(unsigned(bb), 3), threads, 0, st>>>(S, idx, T, off, bb, d, X);
    return cudaGetLastError();
}

cudaError_t mlp_adam4(float *const W[4], const float *const G[4], const int parts[4], float *const M[4],
                      float *const V[4], const int64_t count[4], float lr, int step, cudaStream_t st, int *launches) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, float(step)), c2 = 1.0f - powf(b2, float(step));
    AdamGroups a{};
    int64_t most = 1;
    for (int g = 0; g < 4; ++g) {
        a.W[g] = W[g]; a.G[g] = G[g]; a.M[g] = M[g]; a.V[g] = V[g]; a.count[g] = count[g]; a.parts[g] = parts[g];
        most = count[g] > most ? count[g] : most;
    }
    int64_t blocks = (most + 255) / 256;
    if (blocks > 1024) blocks = 1024;
    if (launches) *launches += 1;
    adam_groups_kernel<<<dim3(unsigned(blocks), 4), 256, 0, st>>>(a, lr, b1, b2, 1e-8f, c1, c2);
    return cudaGetLastError();
}

}  // namespace ssg
