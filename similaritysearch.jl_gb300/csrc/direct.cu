// direct.cu -- exact FP32 scan kernels with a fused bounded top-k.
//
// Replaces the hot loop of search(::ExhaustiveSearch)
// (src/exact/sequential-exhaustive.jl:73-76): for every query, evaluate the
// distance to every database row and keep the k best in KnnSorted order.
// The distance is summed in index order with one FMA per element
// (SqL2: m = x_i - q_i; d = fma(m, m, d), src/dist/vecs.jl:93-102;
//  NormCosine/IP/Cosine: d = fma(x_i, q_i, d), src/dist/cos.jl:78-84),
// so each value is bit-identical to the oracle's sequential sum and within
// the reference's own @simd reassociation tolerance.
//
// Block = QPB threads = QPB queries (one per thread).  Database rows stream
// through shared memory in tiles of TN rows x KC dims; each thread keeps TN
// accumulators and, after the last chunk of a tile, pushes the TN distances
// into its private max-heap (the top-k), pre-filtered against the frontier.
#include "common.cuh"
#include "kernels.h"

#include <cuda_fp16.h>
#include <algorithm>
#include <cmath>

namespace ssg {

namespace {

constexpr int TN = 32;  // database rows per tile (accumulators per thread)
constexpr int KC = 32;  // dims per shared-memory chunk
constexpr int kBufCap = 12;      // buffered top-k: drain checked every 8 values, trigger 4
constexpr int kDrainTrigger = 4;

template <int METRIC>
__device__ __forceinline__ float finish(float acc, float xnorm, float qnorm) {
    if (METRIC == SQL2) return acc;
    if (METRIC == L2) return sqrtf(acc);
    if (METRIC == NORMCOSINE) return 1.0f - acc;
    if (METRIC == IP) return -acc;
    // COSINE: one - dot(a,b) / (norm(a) * norm(b)), a = db row, b = query
    return 1.0f - acc / (xnorm * qnorm);
}

template <int QPB>
__host__ __device__ constexpr size_t direct_static_smem() {
    return size_t(KC) * (QPB + 1) * 4 + size_t(TN) * KC * 4;
}

template <int METRIC, int QPB>
__global__ void __launch_bounds__(QPB)
direct_f32_kernel(ScanArgs a, const float *__restrict__ db, const float *__restrict__ xn,
                  const float *__restrict__ Q, const float *__restrict__ qn, int heap_in_smem) {
    extern __shared__ __align__(16) unsigned char smem[];
    float(*qs)[QPB + 1] = reinterpret_cast<float(*)[QPB + 1]>(smem);
    float(*xs)[KC] = reinterpret_cast<float(*)[KC]>(smem + size_t(KC) * (QPB + 1) * 4);
    uint64_t *hbase = heap_in_smem
        ? reinterpret_cast<uint64_t *>(smem + direct_static_smem<QPB>())
        : a.gheap + (size_t(blockIdx.y) * gridDim.x + blockIdx.x) * size_t(a.kk + kBufCap) * QPB;

    const int t = threadIdx.x;
    const int64_t q0 = int64_t(blockIdx.x) * QPB;
    const int64_t qi = q0 + t;
    const bool qvalid = qi < a.m;
    const int64_t lo = int64_t(blockIdx.y) * a.split_len;
    const int64_t hi = lo + a.split_len < a.n ? lo + a.split_len : a.n;
    const int dim = int(a.dim);

    BufferedTopK T;
    T.init(hbase + t, hbase + size_t(a.kk) * QPB + t, a.kk, QPB);
    const float qnorm = (METRIC == COSINE && qvalid) ? qn[qi] : 1.0f;
    // the query's bound shared with the other splits (ScanArgs::qbound)
    uint32_t *qb = (a.qbound && qvalid) ? a.qbound + qi : nullptr;
    float published = INFINITY;

    for (int64_t j0 = lo; j0 < hi; j0 += TN) {
        float acc[TN];
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[j] = 0.0f;

        for (int kc = 0; kc < dim; kc += KC) {
            __syncthreads();
            for (int e = t; e < QPB * KC; e += QPB) {
                int r = e / KC, c = e % KC;
                int64_t qr = q0 + r;
                float v = 0.0f;
                if (qr < a.m && kc + c < dim) v = Q[qr * dim + kc + c];
                qs[c][r] = v;
            }
            for (int e = t; e < TN * KC; e += QPB) {
                int r = e / KC, c = e % KC;
                int64_t xr = j0 + r;
                float v = 0.0f;
                if (xr < hi && kc + c < dim) v = db[xr * dim + kc + c];
                xs[r][c] = v;
            }
            __syncthreads();
#pragma unroll
            for (int c = 0; c < KC; c += 4) {
                const float qa = qs[c][t], qb = qs[c + 1][t], qc = qs[c + 2][t], qd = qs[c + 3][t];
#pragma unroll
                for (int j = 0; j < TN; ++j) {
                    const float4 x = *reinterpret_cast<const float4 *>(&xs[j][c]);
                    if (METRIC == SQL2 || METRIC == L2) {
                        float m0 = x.x - qa; acc[j] = fmaf(m0, m0, acc[j]);
                        float m1 = x.y - qb; acc[j] = fmaf(m1, m1, acc[j]);
                        float m2 = x.z - qc; acc[j] = fmaf(m2, m2, acc[j]);
                        float m3 = x.w - qd; acc[j] = fmaf(m3, m3, acc[j]);
                    } else {
                        acc[j] = fmaf(x.x, qa, acc[j]);
                        acc[j] = fmaf(x.y, qb, acc[j]);
                        acc[j] = fmaf(x.z, qc, acc[j]);
                        acc[j] = fmaf(x.w, qd, acc[j]);
                    }
                }
            }
        }
        const float bnd = qb ? bound_read(qb) : INFINITY;
        float thr = fminf(T.topd, bnd);
#pragma unroll
        for (int g = 0; g < TN; g += 8) {
#pragma unroll
            for (int j = g; j < g + 8; ++j) {
                const int64_t id = j0 + j;
                if (qvalid && id < hi) {
                    const float d = finish<METRIC>(acc[j], METRIC == COSINE ? xn[id] : 1.0f, qnorm);
                    if (d <= thr) T.append(d, uint32_t(id + a.id_base));
                }
            }
            T.maybe_drain(kDrainTrigger);
            thr = fminf(T.topd, bnd);
        }
        if (qb && T.topd < published) {
            bound_lower(qb, T.topd);
            published = T.topd;
        }
    }
    T.drain();
    Heap &H = T.H;
    if (qvalid) {
        H.sort_ascending();
        uint64_t *out = a.cand + (size_t(qi) * a.splits + blockIdx.y) * a.kk;
        for (int i = 0; i < a.kk; ++i) out[i] = H.h[i * QPB];
    }
}

constexpr size_t kSmemBudget = 200 * 1024;

template <int QPB>
bool heap_fits(int kk) {
    return direct_static_smem<QPB>() + size_t(kk + kBufCap) * QPB * 8 <= kSmemBudget;
}

template <int METRIC, int QPB>
cudaError_t launch_direct_t(const ScanArgs &a, const float *db, const float *xn, const float *q,
                            const float *qn, cudaStream_t st) {
    const bool in_smem = heap_fits<QPB>(a.kk);
    size_t smem = direct_static_smem<QPB>() + (in_smem ? size_t(a.kk + kBufCap) * QPB * 8 : 0);
    auto kern = direct_f32_kernel<METRIC, QPB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    dim3 grid(unsigned((a.m + QPB - 1) / QPB), unsigned(a.splits));
    kern<<<grid, QPB, smem, st>>>(a, db, xn, q, qn, in_smem ? 1 : 0);
    return cudaGetLastError();
}

int direct_qpb(int kk) { return heap_fits<128>(kk) ? 128 : 32; }

}  // namespace

size_t direct_gheap_bytes(const ScanArgs &a) {
    int qpb = direct_qpb(a.kk);
    bool fits = qpb == 128 ? heap_fits<128>(a.kk) : heap_fits<32>(a.kk);
    if (fits) return 0;
    size_t blocks = size_t((a.m + qpb - 1) / qpb) * a.splits;
    return blocks * size_t(a.kk + kBufCap) * qpb * 8;
}

cudaError_t launch_direct_f32(const ScanArgs &a, const float *db, const float *db_norm,
                              const float *q, const float *q_norm, cudaStream_t st, int *launches) {
    const int qpb = direct_qpb(a.kk);
    if (launches) *launches += 1;
#define SSG_DIRECT_CASE(MET)                                                                 \
    case MET:                                                                                \
        return qpb == 128 ? launch_direct_t<MET, 128>(a, db, db_norm, q, q_norm, st)         \
                          : launch_direct_t<MET, 32>(a, db, db_norm, q, q_norm, st);
    switch (a.metric) {
        SSG_DIRECT_CASE(SQL2)
        SSG_DIRECT_CASE(L2)
        SSG_DIRECT_CASE(NORMCOSINE)
        SSG_DIRECT_CASE(COSINE)
        SSG_DIRECT_CASE(IP)
        default: return cudaErrorInvalidValue;
    }
#undef SSG_DIRECT_CASE
}

// ---------------------------------------------------------------------------
// Finalize: merge per-split sorted key lists, cut to k, decode to the
// reference's output form (1-based UInt32 ids, Float32 dists, 0 / Inf32 when
// fewer than k exist -- src/SimilaritySearch.jl:309-313, allknn.jl:43-46).
// ---------------------------------------------------------------------------
namespace {

__global__ void finalize_kernel(FinalizeArgs a, int P) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t *s = reinterpret_cast<uint64_t *>(smem);
    const int64_t j = blockIdx.x;
    const int total = a.segs * a.kk;
    const uint64_t *src = a.cand + size_t(j) * total;
    for (int i = threadIdx.x; i < P; i += blockDim.x) s[i] = i < total ? src[i] : KEY_EMPTY;
    if (a.segs > 1) block_bitonic_sort(s, P);
    else __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t *oi = a.out_ids + size_t(j) * a.k_out;
        float *od = a.out_dists + size_t(j) * a.k_out;
        int w = 0;
        const uint32_t self0 = uint32_t(a.self_ids ? a.self_ids[j] : j + a.self_base);
        bool dropped = !a.exclude_self;
        const int limit = a.k_out + (a.exclude_self ? 1 : 0);
        for (int i = 0; i < limit && i < P && w < a.k_out; ++i) {
            uint64_t key = s[i];
            if (!dropped && key != KEY_EMPTY && key_id0(key) == self0) { dropped = true; continue; }
            if (key == KEY_EMPTY) { oi[w] = 0; od[w] = INFINITY; }
            else { oi[w] = key_id0(key) + 1; od[w] = key_dist(key); }
            ++w;
        }
        for (; w < a.k_out; ++w) { oi[w] = 0; od[w] = INFINITY; }
    }
}

// Merges groups of `group` sorted segments of kk keys into one sorted
// segment of the group's kk smallest keys: the pass used when a query's
// splits x kk candidates exceed one block's shared memory.
__global__ void merge_groups_kernel(const uint64_t *__restrict__ in, int segs, int kk, int group, int out_segs,
                                    int P, uint64_t *__restrict__ out) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t *s = reinterpret_cast<uint64_t *>(smem);
    const int64_t j = blockIdx.x;
    const int g = blockIdx.y;
    const int s0 = g * group;
    const int ns = (segs - s0) < group ? (segs - s0) : group;
    const int total = ns * kk;
    const uint64_t *src = in + (size_t(j) * segs + s0) * kk;
    for (int i = threadIdx.x; i < P; i += blockDim.x) s[i] = i < total ? src[i] : KEY_EMPTY;
    block_bitonic_sort(s, P);
    uint64_t *dst = out + (size_t(j) * out_segs + g) * kk;
    for (int i = threadIdx.x; i < kk; i += blockDim.x) dst[i] = s[i];
}

}  // namespace

cudaError_t launch_merge_groups(const uint64_t *in, int64_t m, int segs, int kk, int group, uint64_t *out,
                                cudaStream_t st, int *launches) {
    const int out_segs = (segs + group - 1) / group;
    const int P = next_pow2(int64_t(group) * kk);
    const size_t smem = size_t(P) * 8;
    cudaError_t e = cudaFuncSetAttribute(merge_groups_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    if (launches) *launches += 1;
    merge_groups_kernel<<<dim3(unsigned(m), unsigned(out_segs)), 256, smem, st>>>(in, segs, kk, group, out_segs, P,
                                                                                  out);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const FinalizeArgs &a, cudaStream_t st, int *launches) {
    const int P = next_pow2(int64_t(a.segs) * a.kk);
    size_t smem = size_t(P) * 8;
    cudaError_t e = cudaFuncSetAttribute(finalize_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(smem));
    if (e != cudaSuccess) return e;
    if (launches) *launches += 1;
    finalize_kernel<<<unsigned(a.m), 256, smem, st>>>(a, P);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Prep kernels.
// ---------------------------------------------------------------------------
namespace {

__global__ void row_norms_kernel(const float *__restrict__ x, int64_t rows, int64_t dim,
                                 float *__restrict__ out) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= rows) return;
    const float *r = x + i * dim;
    float s = 0.0f;
    for (int64_t c = 0; c < dim; ++c) s = fmaf(r[c], r[c], s);
    out[i] = sqrtf(s);
}

template <typename T>
__device__ __forceinline__ float to_f32(T v) { return float(v); }
template <>
__device__ __forceinline__ float to_f32<__half>(__half v) { return __half2float(v); }

// Float32(x) for every element (the Float32 casts of vecs-cast-f32.jl).
template <typename T>
__global__ void cast_kernel(const T *__restrict__ src, int64_t count, float *__restrict__ dst) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (; i < count; i += stride) dst[i] = to_f32<T>(src[i]);
}

__global__ void row_sq_norms_kernel(const float *__restrict__ x, int64_t rows, int64_t dim,
                                    float *__restrict__ out, float *__restrict__ max_out) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    float s = 0.0f;
    if (i < rows) {
        const float *r = x + i * dim;
        for (int64_t c = 0; c < dim; ++c) s = fmaf(r[c], r[c], s);
        out[i] = s;
    }
    // block max, then one atomic per block (non-negative floats order as ints)
    for (int o = 16; o > 0; o >>= 1) s = fmaxf(s, __shfl_xor_sync(0xffffffffu, s, o));
    if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<int *>(max_out), __float_as_int(s));
}

__global__ void gather_rows_kernel(const uint32_t *__restrict__ src, const int64_t *__restrict__ idx,
                                   int64_t count, int64_t words, uint32_t *__restrict__ dst) {
    const int64_t total = count * words;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
         i += int64_t(gridDim.x) * blockDim.x) {
        const int64_t r = i / words, w = i % words;
        dst[i] = src[idx[r] * words + w];
    }
}

__global__ void scatter_results_kernel(const uint32_t *__restrict__ si, const float *__restrict__ sd,
                                       const int64_t *__restrict__ idx, int64_t count, int k,
                                       uint32_t *__restrict__ ids, float *__restrict__ dists) {
    const int64_t total = count * k;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
         i += int64_t(gridDim.x) * blockDim.x) {
        const int64_t r = i / k, c = i % k;
        ids[idx[r] * k + c] = si[i];
        dists[idx[r] * k + c] = sd[i];
    }
}

}  // namespace

cudaError_t launch_row_sq_norms(const float *x, int64_t rows, int64_t dim, float *out, float *max_out,
                                cudaStream_t st, int *launches) {
    if (rows <= 0) return cudaSuccess;
    if (launches) *launches += 1;
    row_sq_norms_kernel<<<unsigned((rows + 255) / 256), 256, 0, st>>>(x, rows, dim, out, max_out);
    return cudaGetLastError();
}

cudaError_t launch_gather_rows(const void *src, const int64_t *idx, int64_t count, size_t row_bytes, void *dst,
                               cudaStream_t st, int *launches) {
    if (count <= 0) return cudaSuccess;
    const int64_t words = int64_t(row_bytes / 4);
    int64_t blocks = std::min<int64_t>((count * words + 255) / 256, 148 * 32);
    if (launches) *launches += 1;
    gather_rows_kernel<<<unsigned(blocks), 256, 0, st>>>(static_cast<const uint32_t *>(src), idx, count, words,
                                                         static_cast<uint32_t *>(dst));
    return cudaGetLastError();
}

// Closest pairs.  Row j of (ids, dists) holds object j of B's kk nearest
// candidates, sorted by (distance, id); pair (ids[j][t], j) gets the key
// (distance, j * kk + t), so a row is a sorted segment of the global order
// (distance, j, rank) and the segment merge yields the k closest pairs.
__global__ void pair_keys_kernel(const uint32_t *__restrict__ ids, const float *__restrict__ dists, int64_t total,
                                 uint64_t *__restrict__ keys) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x)
        keys[i] = ids[i] ? make_key(dists[i], uint32_t(i)) : KEY_EMPTY;
}

// sel_ids / sel_d: the merged top k (1-based flat index + 1, 0 = none)
__global__ void pair_decode_kernel(const uint32_t *__restrict__ sel_ids, const float *__restrict__ sel_d, int k,
                                   const uint32_t *__restrict__ ids, int kk, int32_t *__restrict__ oi,
                                   int32_t *__restrict__ oj, float *__restrict__ od) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= k) return;
    const uint32_t f = sel_ids[r];
    if (f == 0) { oi[r] = 0; oj[r] = 0; od[r] = INFINITY; return; }
    const uint32_t flat = f - 1;
    oi[r] = int32_t(ids[flat]);
    oj[r] = int32_t(flat / uint32_t(kk)) + 1;
    od[r] = sel_d[r];
}

cudaError_t launch_pair_keys(const uint32_t *ids, const float *dists, int64_t total, uint64_t *keys, cudaStream_t st,
                             int *launches) {
    if (total <= 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>((total + 255) / 256, 148 * 32);
    if (launches) *launches += 1;
    pair_keys_kernel<<<unsigned(blocks), 256, 0, st>>>(ids, dists, total, keys);
    return cudaGetLastError();
}

cudaError_t launch_pair_decode(const uint32_t *sel_ids, const float *sel_d, int k, const uint32_t *ids, int kk,
                               int32_t *oi, int32_t *oj, float *od, cudaStream_t st, int *launches) {
    if (k <= 0) return cudaSuccess;
    if (launches) *launches += 1;
    pair_decode_kernel<<<unsigned((k + 127) / 128), 128, 0, st>>>(sel_ids, sel_d, k, ids, kk, oi, oj, od);
    return cudaGetLastError();
}

cudaError_t launch_scatter_results(const uint32_t *src_ids, const float *src_d, const int64_t *idx, int64_t count,
                                   int k, uint32_t *ids, float *dists, cudaStream_t st, int *launches) {
    if (count <= 0) return cudaSuccess;
    int64_t blocks = std::min<int64_t>((count * k + 255) / 256, 148 * 32);
    if (launches) *launches += 1;
    scatter_results_kernel<<<unsigned(blocks), 256, 0, st>>>(src_ids, src_d, idx, count, k, ids, dists);
    return cudaGetLastError();
}

cudaError_t launch_row_norms(const float *x, int64_t rows, int64_t dim, float *out,
                             cudaStream_t st, int *launches) {
    if (rows <= 0) return cudaSuccess;
    if (launches) *launches += 1;
    row_norms_kernel<<<unsigned((rows + 255) / 256), 256, 0, st>>>(x, rows, dim, out);
    return cudaGetLastError();
}

cudaError_t launch_cast_f32(const void *src, int elem, int64_t count, float *dst, cudaStream_t st,
                            int *launches) {
    if (count <= 0) return cudaSuccess;
    int64_t blocks = (count + 255) / 256;
    if (blocks > 65535 * 16) blocks = 65535 * 16;
    if (launches) *launches += 1;
    switch (elem) {
        case 2: cast_kernel<double><<<unsigned(blocks), 256, 0, st>>>((const double *)src, count, dst); break;
        case 3: cast_kernel<__half><<<unsigned(blocks), 256, 0, st>>>((const __half *)src, count, dst); break;
        case 4: cast_kernel<uint8_t><<<unsigned(blocks), 256, 0, st>>>((const uint8_t *)src, count, dst); break;
        case 5: cast_kernel<int8_t><<<unsigned(blocks), 256, 0, st>>>((const int8_t *)src, count, dst); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace ssg
