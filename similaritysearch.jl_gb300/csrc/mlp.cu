// mlp.cu -- kernels of the learned shortlist: a small MLP (d -> H (ReLU) -> E)
// trained with a triplet loss, forward and backward written by hand.
//
// The GEMMs are small (H = 256, E = 64) and off the search's hot path, so
// they are SIMT kernels: 64 x 64 output tiles, 4 x 4 per thread, FP32
// accumulation.  With `bf16` set, every operand element is rounded to BF16
// as it is staged (the BF16-operand / FP32-accumulate arithmetic of the
// tensor cores); weights are kept in FP32 (master copy) and updated by Adam.
#include "kernels.h"

#include <cuda_bf16.h>

namespace ssg {

namespace {

constexpr int GT = 64;   // output tile
constexpr int GK = 16;   // k per stage

__device__ __forceinline__ float round_bf16(float v, int bf16) {
    return bf16 ? __bfloat162float(__float2bfloat16_rn(v)) : v;
}

// C[M x N] = op(A) * op(B) (+ bias[n]) (ReLU?)
//   op(A) = A (M x K, row-major) or A^T (A stored K x M) when ta
//   op(B) = B^T (B stored N x K)  or B   (B stored K x N) when tb
__global__ void __launch_bounds__(256) mlp_gemm_kernel(const float *__restrict__ A, const float *__restrict__ B,
                                                        const float *__restrict__ bias, float *__restrict__ Cm,
                                                        int M, int N, int K, int ta, int tb, int relu, int bf16,
                                                        int accumulate) {
    __shared__ float sA[GK][GT + 1];
    __shared__ float sB[GK][GT + 1];
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    const int m0 = blockIdx.y * GT, n0 = blockIdx.x * GT;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += GK) {
        // consecutive threads walk the operand's contiguous dimension: K for
        // a row-major operand, the rows for a transposed one (coalesced)
        for (int e = tid; e < GK * GT; e += 256) {
            {
                const int kk = ta ? e / GT : e % GK, r = ta ? e % GT : e / GK;
                const int gm = m0 + r, gk = k0 + kk;
                float va = 0.0f;
                if (gm < M && gk < K) va = ta ? A[size_t(gk) * M + gm] : A[size_t(gm) * K + gk];
                sA[kk][r] = round_bf16(va, bf16);
            }
            {
                const int kk = tb ? e / GT : e % GK, r = tb ? e % GT : e / GK;
                const int gn = n0 + r, gk = k0 + kk;
                float vb = 0.0f;
                if (gn < N && gk < K) vb = tb ? B[size_t(gk) * N + gn] : B[size_t(gn) * K + gk];
                sB[kk][r] = round_bf16(vb, bf16);
            }
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = sA[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = sB[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int gm = m0 + ty * 4 + i;
        if (gm >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int gn = n0 + tx * 4 + j;
            if (gn >= N) continue;
            float v = acc[i][j];
            if (bias) v += bias[gn];
            if (relu) v = fmaxf(v, 0.0f);
            float *c = Cm + size_t(gm) * N + gn;
            *c = accumulate ? *c + v : v;
        }
    }
}

// Triplet loss on Z = [anchors; positives; negatives] (3B rows of E):
// l = max(0, |a-p|^2 - |a-n|^2 + margin), mean over the batch; writes dL/dZ.
__global__ void triplet_kernel(const float *__restrict__ Z, int B, int E, float margin, float *__restrict__ dZ,
                               float *__restrict__ loss_sum, int *__restrict__ active) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const float *za = Z + size_t(b) * E;
    const float *zp = Z + size_t(B + b) * E;
    const float *zn = Z + size_t(2 * B + b) * E;
    float dp = 0.0f, dn = 0.0f;
    for (int e = 0; e < E; ++e) {
        const float u = za[e] - zp[e], w = za[e] - zn[e];
        dp = fmaf(u, u, dp);
        dn = fmaf(w, w, dn);
    }
    const float l = dp - dn + margin;
    float *ga = dZ + size_t(b) * E;
    float *gp = dZ + size_t(B + b) * E;
    float *gn = dZ + size_t(2 * B + b) * E;
    const float s = 2.0f / float(B);
    if (l > 0.0f) {
        atomicAdd(loss_sum, l / float(B));
        atomicAdd(active, 1);
        for (int e = 0; e < E; ++e) {
            ga[e] = s * (zn[e] - zp[e]);
            gp[e] = -s * (za[e] - zp[e]);
            gn[e] = s * (za[e] - zn[e]);
        }
    } else {
        for (int e = 0; e < E; ++e) { ga[e] = 0.0f; gp[e] = 0.0f; gn[e] = 0.0f; }
    }
}

// dH *= (H > 0)
__global__ void relu_backward_kernel(float *__restrict__ dH, const float *__restrict__ H, int64_t count) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x)
        if (!(H[i] > 0.0f)) dH[i] = 0.0f;
}

// out[n] = sum over rows of G[row][n]
__global__ void colsum_kernel(const float *__restrict__ G, int rows, int N, float *__restrict__ out) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.0f;
    for (int r = 0; r < rows; ++r) s += G[size_t(r) * N + n];
    out[n] = s;
}

__global__ void adam_kernel(float *__restrict__ W, const float *__restrict__ G, float *__restrict__ Mo,
                            float *__restrict__ Vo, int64_t count, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count;
         i += int64_t(gridDim.x) * blockDim.x) {
        const float g = G[i];
        const float m = b1 * Mo[i] + (1.0f - b1) * g;
        const float v = b2 * Vo[i] + (1.0f - b2) * g * g;
        Mo[i] = m;
        Vo[i] = v;
        W[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
    }
}

}  // namespace

cudaError_t mlp_gemm(const float *A, const float *B, const float *bias, float *C, int M, int N, int K, int ta, int tb,
                     int relu, int bf16, int accumulate, cudaStream_t st, int *launches) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    dim3 grid(unsigned((N + GT - 1) / GT), unsigned((M + GT - 1) / GT));
    if (launches) *launches += 1;
    mlp_gemm_kernel<<<grid, 256, 0, st>>>(A, B, bias, C, M, N, K, ta, tb, relu, bf16, accumulate);
    return cudaGetLastError();
}

cudaError_t mlp_triplet(const float *Z, int B, int E, float margin, float *dZ, float *loss_sum, int *active,
                        cudaStream_t st, int *launches) {
    if (launches) *launches += 1;
    triplet_kernel<<<unsigned((B + 127) / 128), 128, 0, st>>>(Z, B, E, margin, dZ, loss_sum, active);
    return cudaGetLastError();
}

cudaError_t mlp_relu_backward(float *dH, const float *H, int64_t count, cudaStream_t st, int *launches) {
    if (launches) *launches += 1;
    int64_t blocks = (count + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    relu_backward_kernel<<<unsigned(blocks), 256, 0, st>>>(dH, H, count);
    return cudaGetLastError();
}

cudaError_t mlp_colsum(const float *G, int rows, int N, float *out, cudaStream_t st, int *launches) {
    if (launches) *launches += 1;
    colsum_kernel<<<unsigned((N + 127) / 128), 128, 0, st>>>(G, rows, N, out);
    return cudaGetLastError();
}

cudaError_t mlp_adam(float *W, const float *G, float *M, float *V, int64_t count, float lr, int step,
                     cudaStream_t st, int *launches) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, float(step)), c2 = 1.0f - powf(b2, float(step));
    if (launches) *launches += 1;
    int64_t blocks = (count + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    adam_kernel<<<unsigned(blocks), 256, 0, st>>>(W, G, M, V, count, lr, b1, b2, 1e-8f, c1, c2);
    return cudaGetLastError();
}

}  // namespace ssg
