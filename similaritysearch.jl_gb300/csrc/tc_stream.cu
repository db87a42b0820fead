// tc_stream.cu -- tensor-core distance tiles for wide vectors, BF16 or FP8.
//
// The reduced-precision methods for any dimension: like tc_bf16.cu, but both
// operands stream through shared memory one K-block at a time, so a 768-wide
// query tile does not have to stay on chip.  Operands are BF16 or FP8 e4m3
// with one scale per vector (x ~= s_x * x8, s_x = max|x_i| / 448); the
// tensor cores accumulate in FP32 (tcgen05.mma kind::f16 / kind::f8f6f4) and
// the epilogue turns the raw dot v into an approximate distance
//      d~ = fma(v * gamma_q, alpha_x, beta_x)
// with per-query gamma (the query's scale) and per-row alpha / beta:
//      IP, NormCosine:  alpha = -s_x,              beta = 0
//      Cosine:          alpha = -s_x / |x|,        beta = 0
//      SqL2, L2:        alpha = -2 s_x,            beta = |x|^2
// which ranks like the exact metric.  kk = overfetch * k candidates per query
// survive into the exact FP32 rerank (finalize_rerank_kernel).
//
// Layout in HBM: tiles of 128 rows; each tile is a sequence of K-blocks of
// 128 bytes per row (64 BF16 or 128 FP8 elements) with the 128-byte swizzle
// applied, so one K-block of a query tile and one of a database tile (16 KB
// each) form one pipeline stage, fetched with two TMA bulk copies.
//
// Roles per CTA (one 128-query tile): warp 0 TMA producer, warp 1 TMEM owner
// and MMA issuer (double-buffered 128 x 128 FP32 accumulators), 4 * CS
// epilogue warps (CS warps share each TMEM lane quarter and split the
// columns).  Every wait is bounded (tc_ptx.cuh).
#include "common.cuh"
#include "kernels.h"
#include "tc_ptx.cuh"

#include <cuda_bf16.h>
#include <cuda_fp8.h>

namespace ssg {

namespace {

constexpr int TILE = 128;
constexpr int SWB = 128;                      // bytes per swizzled K-block row
constexpr int KBLOCK_BYTES = TILE * SWB;      // 16 KB per operand per K-block
constexpr int kBufCap = 12;
constexpr int kDrainTrigger = 4;
// TMEM accumulators (128 columns each): all 512 columns, so the MMAs run up
// to three tiles ahead of the epilogue
constexpr int NACC = 4;

template <int CS>
__host__ __device__ constexpr int st_threads() { return 64 + TILE * CS; }

// ---------------------------------------------------------------------------
// Prep: rows -> swizzled K-block tiles (BF16 or scaled FP8) + per-row scale.
// One warp per row.
// ---------------------------------------------------------------------------
// split != 0 (BF16 only): the plain method's two-piece form, three segments
// of kp = kbytes / 6 elements along K, database rows (split 1) as
// [lo | hi | hi] and query rows (split 2) as [hi | lo | hi], with
// hi = bf16(x) and lo = bf16(x - hi) (see tc_bf16.cu, bf16_tile_kernel).
__global__ void stream_tile_kernel(const float *__restrict__ x, int64_t rows, int dim, int kbytes, int fp8,
                                   int split, int64_t tiles, uint8_t *__restrict__ out, float *__restrict__ scale) {
    const int lane = threadIdx.x % 32;
    const int64_t wid = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32;
    const int64_t nw = int64_t(gridDim.x) * blockDim.x / 32;
    const int es = fp8 ? 1 : 2;
    const int per_chunk = 16 / es;             // elements per 16-byte chunk
    const int nchunks = kbytes / 16;           // chunks per padded row
    const size_t tile_bytes = size_t(TILE) * kbytes;
    for (int64_t row = wid; row < tiles * TILE; row += nw) {
        const bool valid = row < rows;
        const float *xr = x + (valid ? row : 0) * dim;
        float s = 1.0f;
        if (fp8) {
            float mx = 0.0f;
            if (valid)
                for (int c = lane; c < dim; c += 32) mx = fmaxf(mx, fabsf(xr[c]));
            for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            s = mx > 0.0f ? mx / 448.0f : 1.0f;
            if (lane == 0) scale[row] = valid ? s : 0.0f;
        }
        const float inv = 1.0f / s;
        const int64_t tile = row / TILE;
        const int r = int(row % TILE);
        for (int ch = lane; ch < nchunks; ch += 32) {
            __align__(16) uint8_t buf[16];
            const int e0 = ch * per_chunk;
            if (fp8) {
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    const float f = (valid && e0 + e < dim) ? xr[e0 + e] * inv : 0.0f;
                    buf[e] = __nv_cvt_float_to_fp8(f, __NV_SATFINITE, __NV_E4M3);
                }
            } else if (split) {
                const int kp = kbytes / 6;
                const int seg = e0 / kp, scol = e0 % kp;
                const bool low = (split == 1 && seg == 0) || (split == 2 && seg == 1);
                __nv_bfloat16 *b = reinterpret_cast<__nv_bfloat16 *>(buf);
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const float f = (valid && scol + e < dim) ? xr[scol + e] : 0.0f;
                    const __nv_bfloat16 hi = __float2bfloat16_rn(f);
                    b[e] = low ? __float2bfloat16_rn(f - __bfloat162float(hi)) : hi;
                }
            } else {
                __nv_bfloat16 *b = reinterpret_cast<__nv_bfloat16 *>(buf);
#pragma unroll
                for (int e = 0; e < 8; ++e) b[e] = __float2bfloat16_rn((valid && e0 + e < dim) ? xr[e0 + e] : 0.0f);
            }
            const int kb = ch / (SWB / 16);
            const uint32_t off = tc::swizzled_offset(uint32_t(r), uint32_t((ch % (SWB / 16)) * 16), SWB);
            uint8_t *dst = out + size_t(tile) * tile_bytes + size_t(kb) * KBLOCK_BYTES + off;
            *reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<const uint4 *>(buf);
        }
    }
}

// alpha / beta per padded database row (see the file comment)
__global__ void stream_coef_kernel(const float *__restrict__ x, int64_t rows, int dim, int64_t padded, int metric,
                                   const float *__restrict__ scale, float *__restrict__ alpha,
                                   float *__restrict__ beta) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= padded) return;
    if (i >= rows) { alpha[i] = 0.0f; beta[i] = 0.0f; return; }
    const float s = scale ? scale[i] : 1.0f;
    float sq = 0.0f;
    if (metric == SQL2 || metric == L2 || metric == COSINE) {
        const float *r = x + i * dim;
        for (int c = 0; c < dim; ++c) sq = fmaf(r[c], r[c], sq);
    }
    if (metric == SQL2 || metric == L2) { alpha[i] = -2.0f * s; beta[i] = sq; }
    else if (metric == COSINE) { alpha[i] = sq > 0.0f ? -s / sqrtf(sq) : 0.0f; beta[i] = 0.0f; }
    else { alpha[i] = -s; beta[i] = 0.0f; }
}

struct StreamArgs {
    const uint8_t *qt, *dt;        // query / database K-block tiles
    const float *alpha, *beta;     // per padded database row
    const float *qgamma;           // per query (FP8 scale) or nullptr (1)
    int64_t n, m;
    int kblocks;                   // K-blocks per tile
    int fp8;
    int kk, splits;
    int heap_rows;                 // query rows of a tile that own heaps (32..128)
    // per query, kBoundWords zero-initialised words of shared pruning bounds
    // (SharedBound), nullptr: unused
    uint32_t *gbound;
    int64_t split_tiles, n_tiles;
    uint64_t *cand;
    int *err;
};

// Heaps exist for the first heap_rows rows of the query tile only: a batch of
// m < 128 queries leaves the rest of its single tile as padding, and the
// shared memory saved goes to deeper copy pipelines.
// Exact pruning bounds shared by all heaps of a query (every split and column
// half of it), kBoundWords words per query, zero-initialised:
//   w[0]      complement of the smallest frontier any full heap reached: that
//             heap alone holds kk keys at or below it;
//   w[1 + j]  at checkpoint j (after 2^j tiles), the largest over the heaps
//             of the c-th best candidate each has seen (c = 1 or 2, all
//             columns counted, filtered or not): once all heaps have
//             published it, kk <= c * heaps candidates lie at or below it;
//   w[8 + j]  how many heaps have published checkpoint j (each publishes its
//             value, fences, then counts; readers read the count, fence,
//             then the value).
// A bound B means the kk-th best approximate distance is <= B, so a
// candidate with d > B can be dropped: the kept set is unchanged.  Small
// batches with long candidate lists scan with ~150 splits whose heaps would
// otherwise each fill up alone; the kernel variant with these bounds
// (BOUND) is used for them only.
constexpr int kCheckpoints = 7;

struct SharedBound {
    uint32_t *w;   // this query's words
    int nheaps;    // heaps per query
    int cbest;     // best-seen values tracked per heap (1 or 2), 0: checkpoints off
    int next_pub, next_read;
    float b1, b2, cap;
    uint32_t top_seen;

    __device__ __forceinline__ void init(uint32_t *words, int heaps, int kk) {
        w = words;
        nheaps = heaps;
        const int c = (kk + heaps - 1) / heaps;
        cbest = c <= 2 ? c : 0;
        next_pub = next_read = 0;
        b1 = b2 = cap = INFINITY;
        top_seen = 0xffffffffu;
    }
    // tightens cap from the frontiers and the completed checkpoints
    __device__ __forceinline__ void refresh() {
        const uint32_t f = ~__ldcg(w);
        if (f < top_seen) {
            top_seen = f;
            cap = fminf(cap, ordered_to_float(f));
        }
        while (cbest && next_read < kCheckpoints) {
            if (__ldcg(w + 8 + next_read) < uint32_t(nheaps)) break;
            __threadfence();
            cap = fminf(cap, ordered_to_float(__ldcg(w + 1 + next_read)));
            ++next_read;
        }
    }
    // a full heap's frontier
    __device__ __forceinline__ void frontier(uint64_t top) {
        const uint32_t o = uint32_t(top >> 32);
        if (o < top_seen) {
            top_seen = o;
            atomicMax(w, ~o);
            cap = fminf(cap, ordered_to_float(o));
        }
    }
    __device__ __forceinline__ void see(float v) {
        if (cbest == 1) {
            b1 = fminf(b1, v);
        } else {
            const float n1 = fminf(b1, v);
            b2 = fminf(b2, fmaxf(b1, v));
            b1 = n1;
        }
    }
    // publishes the checkpoints reached after `done` tiles (all of them once
    // the heap's split is finished)
    __device__ __forceinline__ void checkpoint(int done, bool finished) {
        while (cbest && next_pub < kCheckpoints && (finished || done >= (1 << next_pub))) {
            atomicMax(w + 1 + next_pub, float_to_ordered(cbest == 1 ? b1 : b2));
            __threadfence();
            atomicAdd(w + 8 + next_pub, 1u);
            ++next_pub;
        }
    }
};

template <int CS, int STAGES>
struct StreamSmem {
    static size_t heap_bytes(int kk, int rows) { return size_t(rows) * CS * (kk + kBufCap) * 8; }
    static size_t total(int kk, int rows) {
        return 1024 + size_t(STAGES) * 2 * KBLOCK_BYTES + heap_bytes(kk, rows) + 256;
    }
};

// Epilogue warps of this CTA that own a heap and hold a query: (lane quarter,
// column half) pairs whose quarter starts below heap_rows and below m.  Only
// they take part in the accumulator hand-off; the others leave at once
// instead of spinning on barriers for nothing.
template <int CS>
__device__ __forceinline__ int stream_live_warps(const StreamArgs &a) {
    int live = 0;
    for (int q = 0; q < 4; ++q)
        if (q * 32 < a.heap_rows && int64_t(blockIdx.x) * TILE + q * 32 < a.m) live += CS;
    return live;
}

template <int CS, int STAGES, bool BOUND>
__global__ void __launch_bounds__(st_threads<CS>(), 1) tc_stream_kernel(StreamArgs a) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *sAB = smem;  // [STAGES][A | B]
    uint64_t *heap_base = reinterpret_cast<uint64_t *>(sAB + size_t(STAGES) * 2 * KBLOCK_BYTES);
    uint64_t *buf_base = heap_base + size_t(a.heap_rows) * CS * a.kk;
    uint64_t *bars = buf_base + size_t(a.heap_rows) * CS * kBufCap;
    uint64_t *full = bars;
    uint64_t *empty = full + STAGES;
    uint64_t *acc_full = empty + STAGES;
    uint64_t *acc_empty = acc_full + NACC;
    uint64_t *mma_done = acc_empty + NACC;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);

    constexpr int NCOLS = NACC * TILE;  // all 512 TMEM columns
    const int warp = threadIdx.x / 32;
    const int lane = threadIdx.x % 32;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < NACC; ++b) {
            tc::mbar_init(&acc_full[b], 1);
            tc::mbar_init(&acc_empty[b], stream_live_warps<CS>(a));
        }
        tc::mbar_init(mma_done, 1);
        tc::fence_mbarrier_init();
    }
    if (warp == 1) tc::tmem_alloc<NCOLS>(tmem_slot);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    const int64_t t_lo = int64_t(blockIdx.y) * a.split_tiles;
    int64_t t_hi = t_lo + a.split_tiles;
    if (t_hi > a.n_tiles) t_hi = a.n_tiles;
    const int T_tiles = t_hi > t_lo ? int(t_hi - t_lo) : 0;
    const int KB = a.kblocks;
    const size_t tile_bytes = size_t(KB) * KBLOCK_BYTES;

    if (warp == 0) {
        if (lane == 0) {
            const uint8_t *qtile = a.qt + size_t(blockIdx.x) * tile_bytes;
            int it = 0;
            bool ok = true;
            for (int t = 0; ok && t < T_tiles; ++t) {
                const uint8_t *dtile = a.dt + size_t(t_lo + t) * tile_bytes;
                for (int kb = 0; kb < KB; ++kb, ++it) {
                    const int s = it % STAGES;
                    if (!tc::mbar_wait(&empty[s], ((it / STAGES) & 1) ^ 1, a.err, 11)) { ok = false; break; }
                    tc::mbar_arrive_expect_tx(&full[s], 2 * KBLOCK_BYTES);
                    uint8_t *dst = sAB + size_t(s) * 2 * KBLOCK_BYTES;
                    tc::bulk_g2s(dst, qtile + size_t(kb) * KBLOCK_BYTES, KBLOCK_BYTES, &full[s]);
                    tc::bulk_g2s(dst + KBLOCK_BYTES, dtile + size_t(kb) * KBLOCK_BYTES, KBLOCK_BYTES, &full[s]);
                }
            }
            // wait (bounded) for the copies of the last stages issued
            for (int j = it - STAGES < 0 ? 0 : it - STAGES; j < it; ++j)
                tc::mbar_wait(&full[j % STAGES], (j / STAGES) & 1, a.err, 12);
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = a.fp8 ? tc::idesc_e4m3_f32(TILE, TILE) : tc::idesc_bf16_f32(TILE, TILE);
            const uint32_t base = tc::smem_u32(sAB);
            int it = 0;
            bool ok = true;
            for (int t = 0; ok && t < T_tiles; ++t) {
                const int b = t % NACC;
                if (!tc::mbar_wait(&acc_empty[b], ((t / NACC) & 1) ^ 1, a.err, 13)) break;
                tc::tc_fence_after();
                const uint32_t d_tmem = tmem_base + uint32_t(b * TILE);
                for (int kb = 0; kb < KB; ++kb, ++it) {
                    const int s = it % STAGES;
                    if (!tc::mbar_wait(&full[s], (it / STAGES) & 1, a.err, 14)) { ok = false; break; }
                    tc::tc_fence_after();
                    const uint32_t sa = base + uint32_t(s) * 2 * KBLOCK_BYTES;
                    const uint32_t sb = sa + KBLOCK_BYTES;
#pragma unroll
                    for (int k = 0; k < SWB / 32; ++k) {  // 32 bytes of K per MMA
                        const uint64_t ad = tc::smem_desc(sa + k * 32, SWB);
                        const uint64_t bd = tc::smem_desc(sb + k * 32, SWB);
                        if (a.fp8) tc::mma_f8(d_tmem, ad, bd, idesc, (kb | k) ? 1u : 0u);
                        else tc::mma_f16(d_tmem, ad, bd, idesc, (kb | k) ? 1u : 0u);
                    }
                    tc::mma_commit(&empty[s]);
                }
                if (!ok) break;
                tc::mma_commit(&acc_full[b]);
            }
            tc::mma_commit(mma_done);
            tc::mbar_wait(mma_done, 0, a.err, 15);
        }
        __syncwarp();
    } else {
        const int e = warp - 2;
        const int cs = e / 4;
        const int quarter = warp % 4;
        const int row = quarter * 32 + lane;
        const int64_t query = int64_t(blockIdx.x) * TILE + row;
        const int hs = a.heap_rows * CS;
        constexpr int CHUNKS = TILE / 32 / CS;
        const float gamma = (a.qgamma && query < a.m) ? a.qgamma[query] : 1.0f;
        // padding rows of a partial query tile filter everything out (a
        // -inf threshold), and warps holding only padding rows skip the
        // epilogue: they just hand the accumulator back (they own no heap)
        const bool qvalid = query < a.m;
        const bool warp_live = quarter * 32 < a.heap_rows && int64_t(blockIdx.x) * TILE + quarter * 32 < a.m;
        uint64_t *heap = heap_base + (cs * a.heap_rows + quarter * 32 + lane);
        uint64_t *cbuf = buf_base + (cs * a.heap_rows + quarter * 32 + lane);
        if (warp_live) Heap{heap, a.kk, hs}.init();
        uint64_t top = KEY_EMPTY;
        float topd = qvalid ? INFINITY : -INFINITY;
        const bool shared = BOUND && qvalid;
        SharedBound sb;
        sb.init(shared ? a.gbound + size_t(query) * kBoundWords : nullptr, a.splits * CS, a.kk);
        int nbuf = 0;
        for (int t = 0; warp_live && t < T_tiles; ++t) {
            const int b = t % NACC;
            int ok = 1;
            if (lane == 0) ok = tc::mbar_wait(&acc_full[b], (t / NACC) & 1, a.err, 16) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) break;
            tc::tc_fence_after();
            if (shared) {
                sb.refresh();
                topd = fminf(topd, sb.cap);
            }
            const int64_t row0 = (t_lo + t) * TILE + cs * (TILE / CS);
            uint32_t r[CHUNKS][32];
            __syncwarp();
            const uint32_t tbase =
                tmem_base + (uint32_t(quarter * 32) << 16) + uint32_t(b * TILE + cs * (TILE / CS));
#pragma unroll
            for (int c = 0; c < CHUNKS; ++c) tc::tmem_ld_32x32b_x32_async(tbase + uint32_t(c * 32), r[c]);
            tc::tmem_wait_ld();
            tc::tc_fence_before();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&acc_empty[b]);
#pragma unroll
            for (int c = 0; c < CHUNKS; ++c) {
                const int64_t id0 = row0 + c * 32;
                const float *al = a.alpha + id0;
                const float *be = a.beta + id0;
                float dv[32];
                float gmin[4];
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    dv[j] = fmaf(__uint_as_float(r[c][j]) * gamma, __ldg(al + j), __ldg(be + j));
#pragma unroll
                for (int g = 0; g < 4; ++g) gmin[g] = fmin8(dv + 8 * g);
                const float dmin = fmin3(fmin3(gmin[0], gmin[1], gmin[2]), gmin[3], gmin[3]);
                if (shared && sb.cbest) {
                    // best candidates seen, padding rows of the last tile excluded
                    if (sb.cbest == 1 && id0 + 32 <= a.n) {
                        sb.see(dmin);
                    } else {
#pragma unroll
                        for (int j = 0; j < 32; ++j)
                            if (id0 + j < a.n) sb.see(dv[j]);
                    }
                }
                if (__any_sync(0xffffffffu, dmin <= topd)) {
                    const int lim = int(id0 + 32 <= a.n ? 32 : a.n - id0);  // valid columns
#pragma unroll
                    for (int g = 0; g < 4; ++g) {
                        if (!__any_sync(0xffffffffu, gmin[g] <= topd)) continue;
#pragma unroll
                        for (int j = 8 * g; j < 8 * g + 8; ++j) {
                            // raw append (id, distance bits): the key is made
                            // when the buffer drains, once per candidate
                            cbuf[nbuf * hs] = (uint64_t(uint32_t(id0) + uint32_t(j)) << 32) | __float_as_uint(dv[j]);
                            nbuf += (dv[j] <= topd && j < lim) ? 1 : 0;
                        }
                        if (__any_sync(0xffffffffu, nbuf >= kDrainTrigger)) {
                            top = heap_drain_raw<false>(heap, cbuf, a.kk, hs, nbuf, top);
                            nbuf = 0;
                            topd = !qvalid ? -INFINITY : (top == KEY_EMPTY) ? INFINITY : key_dist(top);
                            if (shared) {
                                if (top != KEY_EMPTY) sb.frontier(top);
                                topd = fminf(topd, sb.cap);
                            }
                        }
                    }
                }
            }
            if (shared) sb.checkpoint(t + 1, false);
        }
        if (shared) sb.checkpoint(T_tiles, true);
        if (warp_live) top = heap_drain_raw<false>(heap, cbuf, a.kk, hs, nbuf, top);
        Heap H{heap, a.kk, hs};
        if (warp_live && query < a.m) {
            H.sort_ascending();
            uint64_t *out = a.cand + ((size_t(query) * a.splits + blockIdx.y) * CS + cs) * a.kk;
            for (int i = 0; i < a.kk; ++i) out[i] = H.h[i * hs];
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc::tc_fence_after();
        tc::tmem_dealloc<NCOLS>(tmem_base);
    }
}

constexpr size_t kMaxSmem = 227 * 1024;

template <int CS, int STAGES>
cudaError_t launch_stream_t(const StreamArgs &a, cudaStream_t st) {
    const size_t smem = StreamSmem<CS, STAGES>::total(a.kk, a.heap_rows);
    auto kern = a.gbound ? tc_stream_kernel<CS, STAGES, true> : tc_stream_kernel<CS, STAGES, false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    dim3 grid(unsigned((a.m + TILE - 1) / TILE), unsigned(a.splits));
    kern<<<grid, st_threads<CS>(), smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace

int stream_kbytes(int64_t dim, int fp8) {
    const int64_t bytes = dim * (fp8 ? 1 : 2);
    return int((bytes + SWB - 1) / SWB * SWB);
}
size_t stream_tile_bytes(int64_t dim, int fp8) { return size_t(TILE) * stream_kbytes(dim, fp8); }

int stream_heap_rows(int64_t m) { return m >= TILE ? TILE : int((m + 31) / 32 * 32); }

// (column splits, stages) for kk candidates and heap_rows rows with heaps, or
// false.  Deeper pipelines first (small batches are bound by HBM latency),
// then two epilogue warps per lane quarter.
bool stream_choose(int kk, int heap_rows, int *cs, int *stages) {
    if (StreamSmem<2, 6>::total(kk, heap_rows) <= kMaxSmem) { *cs = 2; *stages = 6; return true; }
    if (StreamSmem<2, 4>::total(kk, heap_rows) <= kMaxSmem) { *cs = 2; *stages = 4; return true; }
    if (StreamSmem<2, 3>::total(kk, heap_rows) <= kMaxSmem) { *cs = 2; *stages = 3; return true; }
    if (StreamSmem<1, 4>::total(kk, heap_rows) <= kMaxSmem) { *cs = 1; *stages = 4; return true; }
    if (StreamSmem<1, 3>::total(kk, heap_rows) <= kMaxSmem) { *cs = 1; *stages = 3; return true; }
    if (StreamSmem<1, 2>::total(kk, heap_rows) <= kMaxSmem) { *cs = 1; *stages = 2; return true; }
    return false;
}

cudaError_t launch_stream_tiles(const float *x, int64_t rows, int64_t dim, int fp8, int64_t tiles, uint8_t *out,
                                float *scale, cudaStream_t st, int *launches, int split) {
    if (split && fp8) return cudaErrorInvalidValue;
    const int64_t warps = tiles * TILE;
    int64_t blocks = (warps * 32 + 255) / 256;
    if (blocks > 148 * 32) blocks = 148 * 32;
    if (blocks < 1) blocks = 1;
    if (launches) *launches += 1;
    const int kbytes = (split ? 3 : 1) * stream_kbytes(dim, fp8);
    stream_tile_kernel<<<unsigned(blocks), 256, 0, st>>>(x, rows, int(dim), kbytes, fp8, split, tiles, out, scale);
    return cudaGetLastError();
}

cudaError_t launch_stream_coefs(int metric, const float *x, int64_t rows, int64_t dim, int64_t padded,
                                const float *scale, float *alpha, float *beta, cudaStream_t st, int *launches) {
    if (launches) *launches += 1;
    stream_coef_kernel<<<unsigned((padded + 255) / 256), 256, 0, st>>>(x, rows, int(dim), padded, metric, scale,
                                                                       alpha, beta);
    return cudaGetLastError();
}

cudaError_t launch_stream_scan(const uint8_t *q_tiles, const uint8_t *d_tiles, const float *alpha, const float *beta,
                               const float *qgamma, int64_t n, int64_t m, int64_t dim, int fp8, int kk, int splits,
                               int heap_rows, uint32_t *gbound, uint64_t *cand, int *err, cudaStream_t st,
                               int *launches, int *segs_per_split) {
    StreamArgs a{};
    a.qt = q_tiles;
    a.dt = d_tiles;
    a.alpha = alpha;
    a.beta = beta;
    a.qgamma = qgamma;
    a.n = n;
    a.m = m;
    a.kblocks = stream_kbytes(dim, fp8) / SWB;
    a.fp8 = fp8;
    a.kk = kk;
    a.splits = splits;
    a.n_tiles = (n + TILE - 1) / TILE;
    a.split_tiles = (a.n_tiles + splits - 1) / splits;
    a.cand = cand;
    a.err = err;
    if (heap_rows < stream_heap_rows(m) || heap_rows > TILE || heap_rows % 32) return cudaErrorInvalidValue;
    a.heap_rows = heap_rows;
    a.gbound = gbound;
    int cs = 0, stages = 0;
    if (!stream_choose(kk, a.heap_rows, &cs, &stages)) return cudaErrorInvalidValue;
    if (segs_per_split) *segs_per_split = cs;
    if (launches) *launches += 1;
    if (cs == 2) {
        if (stages == 6) return launch_stream_t<2, 6>(a, st);
        return stages == 4 ? launch_stream_t<2, 4>(a, st) : launch_stream_t<2, 3>(a, st);
    }
    if (stages == 4) return launch_stream_t<1, 4>(a, st);
    if (stages == 3) return launch_stream_t<1, 3>(a, st);
    return launch_stream_t<1, 2>(a, st);
}

}  // namespace ssg
