// rerank.cu -- exact re-scoring of candidate lists (rerank!, src/rerank.jl:22-41).
//
// For query j, the ids in row j (1-based; the first 0 ends the list, as in
// the reference) are re-evaluated with the exact distance and the valid prefix
// is sorted.  The reference sorts with sortperm and leaves the order of equal
// distances to Base.sort; here ties are ordered by id, which is one of the
// orders the reference can produce and makes the output deterministic.
#include "common.cuh"
#include "exact.cuh"
#include "kernels.h"

namespace ssg {

namespace {

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

// ---------------------------------------------------------------------------
// Merge the per-split approximate candidates, re-rank them with the exact
// FP32 distance and write the k best in (distance, id) order.
// ---------------------------------------------------------------------------
namespace {

template <int METRIC>
__global__ void finalize_rerank_kernel(FinalizeArgs f, const float *db, const float *db_norm, int64_t dim,
                                       const float *q, const float *q_norm, int P1, int P2) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t *s1 = reinterpret_cast<uint64_t *>(smem);
    uint64_t *s2 = s1 + P1;
    const int64_t j = blockIdx.x;
    const int total = f.segs * f.kk;
    const uint64_t *src = f.cand + size_t(j) * total;
    for (int i = threadIdx.x; i < P1; i += blockDim.x) s1[i] = i < total ? src[i] : KEY_EMPTY;
    if (f.segs > 1) block_bitonic_sort(s1, P1);
    else __syncthreads();
    const int rr = f.rerank ? f.rerank : f.kk;
    for (int i = threadIdx.x; i < P2; i += blockDim.x) {
        uint64_t key = KEY_EMPTY;
        if (i < rr) {
            const uint64_t ak = s1[i];
            if (ak != KEY_EMPTY && int64_t(key_id0(ak)) < f.n_rows) {
                const uint32_t id0 = key_id0(ak);
                const float d = exact_pair<METRIC>(db, int64_t(id0), dim, q, j, db_norm, q_norm);
                key = make_key(d, id0);
            }
        }
        s2[i] = key;
    }
    block_bitonic_sort(s2, P2);
    if (f.check && threadIdx.x == 0) {
        // Completeness of an approximate candidate list.  An object y left
        // out was either dropped by a full heap (or a merge of segments), so
        // its approximate key a(y) is at least that segment's last key, or
        // sits in a segment behind the re-ranked list: a(y) >= a_low =
        // min(last key of every full segment, last re-ranked key).  Its exact
        // FP32 distance D(y) >= a(y) + c - E, where c turns keys into
        // distances and E bounds the approximation and evaluation errors:
        //   check 1 (keys |x|^2 - 2 x.q of SqL2 / L2): c = |q|^2,
        //           E = err_scale (R + |q|)^2, R a bound on |y| for every y
        //           that could rank at or before the take-th candidate:
        //           |y - q|^2 <= D_take (up to the FP32 evaluation's relative
        //           error t^2 = (d + 2) 2^-24 of (|y| + |q|)^2) gives
        //           |y| <= ((1 + t) |q| + sqrt(D_take)) / (1 - t), and
        //           |y| <= sqrt(max |x|^2) always;
        //   check 2 (keys -x.q): c = 1 for NormCosine, 0 for InnerProduct,
        //           E = err_scale sqrt(max |x|^2) |q| + 2^-22;
        //   check 3 (Cosine's keys -x.q / |x|): distances 1 + a / |q|, so
        //           a_low enters as 1 + a_low / |q| and E = err_scale (the
        //           split's c plus the FP32 dot, norms, division and
        //           subtraction, (2 d + 16) 2^-24, all relative to 1).
        // If a_low + c - E exceeds the exact distance of the take-th
        // re-ranked candidate (for L2 its square, widened by 2^-20 so that
        // sqrt rounding cannot tie), y ranks behind it: the list holds the
        // exact top `take`.  Evaluated in double.
        // A list shorter than rr (heaps that a shared bound kept from
        // filling) holds every candidate no heap dropped: a_low is then the
        // full segments' smallest last key alone.  A list that holds every
        // row needs no check; one shorter than `take` cannot be certified.
        const int take = f.k_out + (f.exclude_self ? 1 : 0);
        int nv = 0;
        while (nv < rr && s1[nv] != KEY_EMPTY) ++nv;
        if (int64_t(nv) < f.n_total) {
            uint64_t low = nv == rr ? s1[rr - 1] : KEY_EMPTY;
            for (int sgi = 0; sgi < f.segs; ++sgi) {
                const uint64_t last = src[size_t(sgi) * f.kk + f.kk - 1];
                if (last != KEY_EMPTY && last < low) low = last;
            }
            bool certified = nv >= take && low != KEY_EMPTY;
            const double qs = double(f.q_sq[j]);
            const double xm = sqrt(double(f.max_x_sq));
            double c, E;
            if (f.check == 1) {
                const double r = xm + sqrt(qs);
                c = qs;
                E = double(f.err_scale) * r * r;
            } else if (f.check == 3) {
                c = 1.0;
                E = double(f.err_scale);
            } else {
                c = METRIC == NORMCOSINE ? 1.0 : 0.0;
                E = double(f.err_scale) * xm * sqrt(qs) + 2.384185791015625e-7;
            }
            double dtake = certified ? double(key_dist(s2[take - 1])) : 0.0;
            if (METRIC == L2) dtake = dtake * dtake * (1.0 + 9.5367431640625e-7);
            if (f.check == 1 && dtake >= 0.0) {
                const double t = sqrt(double(dim + 2) * 5.9604644775390625e-8);
                const double r = fmin(xm, ((1.0 + t) * sqrt(qs) + sqrt(dtake)) / (1.0 - t)) + sqrt(qs);
                E = double(f.err_scale) * r * r;
            }
            const double a_low = f.check == 3 ? double(key_dist(low)) / sqrt(qs) : double(key_dist(low));
            const double lower = certified ? a_low + c - E : 0.0;
            if (!certified || !(lower > dtake)) {
                f.flags[j] = 1;
                atomicAdd(f.flag_count, 1);
            }
        }
    }
    if (threadIdx.x == 0) {
        uint32_t *oi = f.out_ids + size_t(j) * f.k_out;
        float *od = f.out_dists + size_t(j) * f.k_out;
        int w = 0;
        const uint32_t self0 = uint32_t(f.self_ids ? f.self_ids[j] : j + f.self_base);
        bool dropped = !f.exclude_self;
        const int limit = f.k_out + (f.exclude_self ? 1 : 0);
        for (int i = 0; i < limit && i < P2 && w < f.k_out; ++i) {
            const uint64_t key = s2[i];
            if (!dropped && key != KEY_EMPTY && key_id0(key) == self0) { dropped = true; continue; }
            if (key == KEY_EMPTY) { oi[w] = 0; od[w] = INFINITY; }
            else { oi[w] = key_id0(key) + 1; od[w] = key_dist(key); }
            ++w;
        }
        for (; w < f.k_out; ++w) { oi[w] = 0; od[w] = INFINITY; }
    }
}

}  // namespace

cudaError_t launch_finalize_rerank(int metric, const FinalizeArgs &f, const float *db, const float *db_norm,
                                   int64_t dim, const float *q, const float *q_norm, cudaStream_t st,
                                   int *launches) {
    const int P1 = next_pow2(int64_t(f.segs) * f.kk);
    const int rr = f.rerank ? f.rerank : f.kk;
    if (rr > f.segs * f.kk) return cudaErrorInvalidValue;
    const int P2 = next_pow2(rr);
    const size_t smem = size_t(P1 + P2) * 8;
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    if (launches) *launches += 1;
#define SSG_FR(MET)                                                                                      \
    case MET: {                                                                                          \
        cudaError_t e = cudaFuncSetAttribute(finalize_rerank_kernel<MET>,                                \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));   \
        if (e != cudaSuccess) return e;                                                                  \
        finalize_rerank_kernel<MET><<<unsigned(f.m), 128, smem, st>>>(f, db, db_norm, dim, q, q_norm, P1, P2); \
        return cudaGetLastError();                                                                       \
    }
    switch (metric) {
        SSG_FR(SQL2)
        SSG_FR(L2)
        SSG_FR(NORMCOSINE)
        SSG_FR(COSINE)
        SSG_FR(IP)
        default: return cudaErrorInvalidValue;
    }
#undef SSG_FR
}

}  // namespace ssg
