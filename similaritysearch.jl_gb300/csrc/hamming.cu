// hamming.cu -- binary Hamming scan with a fused bounded top-k.
//
// Replaces search(::ExhaustiveSearch) over MatrixDatabase{UInt64} sketches
// with Dist.Bits.Hamming: d = Float32(sum_w popcount(x_w xor q_w))
// (src/dist/bits.jl:18-25), pushed into KnnSorted in id order
// (src/exact/sequential-exhaustive.jl:73-76).  Distances are integers, so the
// (distance, id) keys -- and therefore ids, distances and their order -- are
// bit-exact with the reference.
//
// Block = QPB threads, one query per thread; the query's words live in
// registers (zero-padded to WMAX words).  Database sketches stream through
// shared memory in tiles of TN rows, copied 16 bytes at a time (cp.async;
// 8 bytes for odd word counts) and read with 128-bit broadcast loads;
// every thread XORs + popcounts them against its own query and pushes the
// distance into its private max-heap when it beats the frontier.
#include "common.cuh"
#include "kernels.h"

namespace ssg {

namespace {

constexpr int TN = 64;
constexpr int kBufCap = 12;      // buffered top-k: drain checked every 8 values, trigger 4
constexpr int kDrainTrigger = 4;

template <int WMAX, int QPB>
__host__ __device__ constexpr size_t ham_static_smem() {
    return size_t(2) * TN * WMAX * 8;  // two sketch tiles: one computed, one landing
}

// 8-byte asynchronous copy global -> shared, zero-filled when !valid
__device__ __forceinline__ void cp_async8(uint64_t *dst, const uint64_t *src, bool valid) {
    const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src), "r"(valid ? 8 : 0) : "memory");
}

// 16-byte asynchronous copy global -> shared (L2 only), zero-filled when !valid
__device__ __forceinline__ void cp_async16(uint64_t *dst, const uint64_t *src, bool valid) {
    const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}

// tile of TN sketches starting at row j0 (rows >= hi and words >= W are
// zeros).  VEC16: two words per copy, for an even W on a 16-byte aligned
// database (every word pair then starts on a 16-byte boundary).
template <int WMAX, int QPB, bool VEC16>
__device__ __forceinline__ void load_sketches(uint64_t (*xs)[WMAX], const uint64_t *__restrict__ db, int64_t j0,
                                              int64_t hi, int W) {
    if constexpr (VEC16) {
        for (int e = threadIdx.x; e < TN * WMAX / 2; e += QPB) {
            const int r = e / (WMAX / 2), c = 2 * (e % (WMAX / 2));
            const int64_t xr = j0 + r;
            const bool v = xr < hi && c < W;
            cp_async16(&xs[r][c], v ? db + xr * W + c : db, v);
        }
    } else {
        for (int e = threadIdx.x; e < TN * WMAX; e += QPB) {
            const int r = e / WMAX, c = e % WMAX;
            const int64_t xr = j0 + r;
            const bool v = xr < hi && c < W;
            cp_async8(&xs[r][c], v ? db + xr * W + c : db, v);
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

template <int WMAX, int QPB, bool VEC16>
__global__ void __launch_bounds__(QPB)
hamming_kernel(ScanArgs a, const uint64_t *__restrict__ db, const uint64_t *__restrict__ Q,
               int heap_in_smem) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t(*xbuf)[WMAX] = reinterpret_cast<uint64_t(*)[WMAX]>(smem);  // [2 * TN][WMAX]
    uint64_t *hbase = heap_in_smem
        ? reinterpret_cast<uint64_t *>(smem + ham_static_smem<WMAX, QPB>())
        : a.gheap + (size_t(blockIdx.y) * gridDim.x + blockIdx.x) * size_t(a.kk + kBufCap) * QPB;

    const int t = threadIdx.x;
    const int W = int(a.dim);
    const int64_t qi = int64_t(blockIdx.x) * QPB + t;
    const bool qvalid = qi < a.m;
    const int64_t lo = int64_t(blockIdx.y) * a.split_len;
    const int64_t hi = lo + a.split_len < a.n ? lo + a.split_len : a.n;

    uint64_t q[WMAX];
#pragma unroll
    for (int w = 0; w < WMAX; ++w) q[w] = (qvalid && w < W) ? Q[qi * W + w] : 0ull;

    BufferedTopK T;
    T.init(hbase + t, hbase + size_t(a.kk) * QPB + t, a.kk, QPB);
    // the query's bound shared with the other splits (ScanArgs::qbound)
    uint32_t *qb = (a.qbound && qvalid) ? a.qbound + qi : nullptr;
    float published = INFINITY;

    if (lo < hi) load_sketches<WMAX, QPB, VEC16>(xbuf, db, lo, hi, W);
    for (int64_t j0 = lo, it = 0; j0 < hi; j0 += TN, ++it) {
        // the next tile lands while this one is scanned
        if (j0 + TN < hi) {
            load_sketches<WMAX, QPB, VEC16>(xbuf + ((it + 1) & 1) * TN, db, j0 + TN, hi, W);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncthreads();
        uint64_t(*xs)[WMAX] = xbuf + (it & 1) * TN;
        const int jn = hi - j0 < TN ? int(hi - j0) : TN;
        const float bnd = qb ? bound_read(qb) : INFINITY;
        float thr = qvalid ? fminf(T.topd, bnd) : -INFINITY;
        for (int g = 0; g < jn; g += 8) {
            // eight rows at once: eight independent XOR + POPC chains per
            // thread (rows past the end are zero words, filtered below)
            int d[8];
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) d[jj] = 0;
#pragma unroll
            for (int w = 0; w < WMAX; w += 2) {
#pragma unroll
                for (int jj = 0; jj < 8; ++jj) {
                    const ulonglong2 x = *reinterpret_cast<const ulonglong2 *>(&xs[g + jj][w]);
                    d[jj] += __popcll(q[w] ^ x.x) + __popcll(q[w + 1] ^ x.y);
                }
            }
            int dmin = d[0];
#pragma unroll
            for (int jj = 1; jj < 8; ++jj) dmin = min(dmin, d[jj]);
            if (!__any_sync(0xffffffffu, float(dmin) <= thr)) continue;
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) {
                const float fd = float(d[jj]);
                if (qvalid && g + jj < jn && fd <= thr) T.append(fd, uint32_t(j0 + g + jj + a.id_base));
            }
            T.maybe_drain(kDrainTrigger);
            if (qvalid) thr = fminf(T.topd, bnd);
        }
        if (qb && T.topd < published) {
            bound_lower(qb, T.topd);
            published = T.topd;
        }
        __syncthreads();  // this buffer is refilled two tiles later
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

template <int WMAX, int QPB>
bool ham_heap_fits(int kk) {
    return ham_static_smem<WMAX, QPB>() + size_t(kk + kBufCap) * QPB * 8 <= kSmemBudget;
}

// Queries per block: long candidate lists fill shared memory with heaps, so
// 64-query blocks (three per SM, six warps) then hide latencies better than
// one 128-query block (four warps).
template <int WMAX>
int ham_qpb(int kk) {
    if (kk >= 48 && ham_heap_fits<WMAX, 64>(kk)) return 64;
    return ham_heap_fits<WMAX, 128>(kk) ? 128 : 32;
}

template <int WMAX, int QPB>
cudaError_t launch_ham_t(const ScanArgs &a, const uint64_t *db, const uint64_t *q, cudaStream_t st) {
    const bool in_smem = ham_heap_fits<WMAX, QPB>(a.kk);
    size_t smem = ham_static_smem<WMAX, QPB>() + (in_smem ? size_t(a.kk + kBufCap) * QPB * 8 : 0);
    // 16-byte copies need every word pair 16-byte aligned: an even W and an
    // aligned base (the library's own buffers are; caller buffers may not be)
    const bool vec16 = (a.dim % 2 == 0) && (reinterpret_cast<uintptr_t>(db) % 16 == 0);
    auto kern = vec16 ? hamming_kernel<WMAX, QPB, true> : hamming_kernel<WMAX, QPB, false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    dim3 grid(unsigned((a.m + QPB - 1) / QPB), unsigned(a.splits));
    kern<<<grid, QPB, smem, st>>>(a, db, q, in_smem ? 1 : 0);
    return cudaGetLastError();
}

template <int WMAX>
cudaError_t launch_ham_w(const ScanArgs &a, const uint64_t *db, const uint64_t *q, cudaStream_t st) {
    const int qpb = ham_qpb<WMAX>(a.kk);
    if (qpb == 128) return launch_ham_t<WMAX, 128>(a, db, q, st);
    if (qpb == 64) return launch_ham_t<WMAX, 64>(a, db, q, st);
    return launch_ham_t<WMAX, 32>(a, db, q, st);
}

template <int WMAX>
size_t ham_gheap(const ScanArgs &a) {
    int qpb = ham_qpb<WMAX>(a.kk);
    bool fits = qpb == 128 ? ham_heap_fits<WMAX, 128>(a.kk)
                           : (qpb == 64 ? ham_heap_fits<WMAX, 64>(a.kk) : ham_heap_fits<WMAX, 32>(a.kk));
    if (fits) return 0;
    return size_t((a.m + qpb - 1) / qpb) * a.splits * size_t(a.kk + kBufCap) * qpb * 8;
}

}  // namespace

size_t hamming_gheap_bytes(const ScanArgs &a) {
    if (a.dim <= 2) return ham_gheap<2>(a);
    if (a.dim <= 4) return ham_gheap<4>(a);
    if (a.dim <= 8) return ham_gheap<8>(a);
    if (a.dim <= 16) return ham_gheap<16>(a);
    return ham_gheap<32>(a);
}

cudaError_t launch_hamming(const ScanArgs &a, const uint64_t *db, const uint64_t *q,
                           cudaStream_t st, int *launches) {
    if (a.dim > 32) return cudaErrorInvalidValue;
    if (launches) *launches += 1;
    if (a.dim <= 2) return launch_ham_w<2>(a, db, q, st);
    if (a.dim <= 4) return launch_ham_w<4>(a, db, q, st);
    if (a.dim <= 8) return launch_ham_w<8>(a, db, q, st);
    if (a.dim <= 16) return launch_ham_w<16>(a, db, q, st);
    return launch_ham_w<32>(a, db, q, st);
}

}  // namespace ssg
