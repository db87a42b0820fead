// tc_bf16.cu -- BF16 tensor-core distance tiles with a fused top-k (tcgen05).
//
// The reduced-precision method: distances between a tile of queries and a
// tile of database rows are computed as one GEMM-shaped contraction on the
// 5th-generation tensor cores (tcgen05.mma kind::f16, BF16 operands, FP32
// accumulators in TMEM), turned into an approximate distance in the epilogue
// and pushed into a per-query bounded top-k of kk = overfetch * k candidates.
// The distance matrix never reaches HBM.  The candidates are then re-ranked
// with the exact FP32 difference-form distance (finalize_rerank_kernel), so
// the reported distances are the plain method's and the ids are exact
// whenever the true neighbours survive the BF16 over-fetch.
//
// Data layout.  Queries and database rows are stored in HBM already in the
// tensor core's operand layout: tiles of 128 rows, split along K into blocks
// of 32 BF16 (64-byte rows) with the 64-byte swizzle applied, so one TMA bulk
// copy (cp.async.bulk) of a tile lands in shared memory ready for the MMA --
// no tensor map and no reformatting on chip.
//
// Two scans share this layout: tc_wide_kernel (heap mode, 128 x 256 MMAs
// over a ring of database K-blocks; the default) and tc_scan_kernel (128 x
// 128 tiles: the threshold filter, the "wide" = 0 setting and the locality
// order's pivot scan).  allknn may scan the database in a locality order
// (rows grouped by nearest pivot; see launch_locality_order).
//
// CTA roles (one 128-row query tile, 320 threads):
//   warp 0      TMA producer: the query tile once, then database tiles (or
//               K-blocks of two tiles) through a ring;
//   warp 1      owns TMEM (four 128 x 128 FP32 accumulators, two 128 x 256
//               in the wide scan, two 128 x 128 for the filter) and issues
//               the MMAs from one thread; the accumulators rotate so the
//               epilogue of one tile overlaps the MMAs of the next;
//   warps 2..9  epilogue, two warps per TMEM lane quarter, each with half of
//               a tile's columns: thread = one query row = one TMEM lane;
//               reads its row 32 columns at a time (tcgen05.ld 32x32b.x32),
//               filters against its heap frontier (or the filter's bound)
//               and keeps its own top-kk heap in shared memory
//               (ChunkTopK).
// Every mbarrier wait is bounded (tc_ptx.cuh); a timeout sets *err and all
// roles unwind, wait for their own in-flight copies/MMAs, free TMEM and exit.
#include "common.cuh"
#include "exact.cuh"
#include "kernels.h"
#include "tc_ptx.cuh"

#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>

namespace ssg {

namespace {

constexpr int TILE = 128;      // rows per query / database tile
constexpr int SW = 64;         // bytes per swizzled K-block row (32 BF16)
constexpr int KBE = SW / 2;    // BF16 elements per K-block

enum { MC_DOT = 0, MC_SQ = 1, MC_COS = 2 };

// Per-thread candidate buffer in front of the heap: drains are checked after
// every 8 columns with a trigger of 4, so at most 3 + 8 entries are pending.
constexpr int kBufCap = 12;
constexpr int kDrainTrigger = 4;

// Column splits of the epilogue: with one query tile per CTA, two warps share
// each TMEM lane quarter and filter half of the tile's columns each (two heaps
// per query, merged later), so every scheduler has two epilogue warps to
// overlap latencies.
template <int QT>
__host__ __device__ constexpr int col_splits() { return QT == 1 ? 2 : 1; }
template <int QT>
__host__ __device__ constexpr int tc_threads() { return 64 + TILE * QT * col_splits<QT>(); }

// TMEM accumulators per query tile: 4 x 128 columns with one query tile per
// CTA (all 512 columns), so the MMAs run up to three tiles ahead of the
// epilogue; 2 with two query tiles, and for the threshold filter, whose
// CTAs may share an SM.  A CTA holding all 512 columns is given enough
// shared memory to be alone on its SM (tcgen05.alloc would otherwise wait
// for the other CTA to finish).
template <int QT, bool FILTER>
__host__ __device__ constexpr int acc_buffers() { return (QT == 1 && !FILTER) ? 4 : 2; }
constexpr size_t kAloneSmem = 120 * 1024;

int metric_class(int metric) {
    if (metric == SQL2 || metric == L2) return MC_SQ;
    if (metric == COSINE) return MC_COS;
    return MC_DOT;
}

// ---------------------------------------------------------------------------
// Prep: FP32 rows -> BF16 tiles in the swizzled operand layout.
// ---------------------------------------------------------------------------
// Tile row i holds source row map[i] when a map is given (a reordering of the
// database), row i otherwise.  split != 0: the two-piece form of the plain
// method on the tensor cores -- each element x as hi = bf16(x) and
// lo = bf16(x - hi), laid out along K in three segments of kp: database rows
// (split 1) as [lo | hi | hi], query rows (split 2) as [hi | lo | hi], so one
// product over K = 3 kp accumulates lo.hi + hi.lo + hi.hi, the two small
// terms first (while the accumulator, and so its rounding, is small).
__global__ void bf16_tile_kernel(const float *__restrict__ x, int64_t rows, int dim, int kp, int split, int64_t tiles,
                                 const uint32_t *__restrict__ map, uint8_t *__restrict__ out) {
    const int kout = split ? 3 * kp : kp;
    const int chunks_per_row = kout / 8;
    const int64_t total = tiles * TILE * chunks_per_row;
    const size_t tile_bytes = size_t(TILE) * kout * 2;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
         i += int64_t(gridDim.x) * blockDim.x) {
        const int cidx = int(i % chunks_per_row);
        const int64_t grow = i / chunks_per_row;
        const int64_t tile = grow / TILE;
        const int r = int(grow % TILE);
        const int col0 = cidx * 8;             // column of the tile (kp is a multiple of 8)
        const int seg = col0 / kp, scol = col0 % kp;
        const bool low = (split == 1 && seg == 0) || (split == 2 && seg == 1);
        __align__(16) __nv_bfloat16 v[8];
        const int64_t src = grow < rows && map ? int64_t(map[grow]) : grow;
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            float f = 0.0f;
            if (grow < rows && scol + e < dim) f = x[src * dim + scol + e];
            const __nv_bfloat16 hi = __float2bfloat16_rn(f);
            v[e] = low ? __float2bfloat16_rn(f - __bfloat162float(hi)) : hi;
        }
        const int blk = col0 / KBE;
        const uint32_t off = tc::swizzled_offset(uint32_t(r), uint32_t((col0 % KBE) * 2), SW);
        uint8_t *dst = out + size_t(tile) * tile_bytes + size_t(blk) * TILE * SW + off;
        *reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<const uint4 *>(v);
    }
}

// Per padded row: |x|^2 (MC_SQ) or 1/|x| (MC_COS), 0 for padding rows.
__global__ void tc_norm_kernel(const float *__restrict__ x, int64_t rows, int dim, int64_t padded, int mc,
                               const uint32_t *__restrict__ map, float *__restrict__ out) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= padded) return;
    float s = 0.0f;
    if (i < rows) {
        const float *r = x + (map ? int64_t(map[i]) : i) * dim;
        for (int c = 0; c < dim; ++c) s = fmaf(r[c], r[c], s);
    }
    out[i] = (mc == MC_COS) ? (s > 0.0f ? 1.0f / sqrtf(s) : 0.0f) : s;
}

// ---------------------------------------------------------------------------
// The scan.
// ---------------------------------------------------------------------------
struct TcArgs {
    const uint8_t *qt;      // query tiles
    const uint8_t *dt;      // database tiles
    const float *dnorm;     // per padded database row (MC_SQ / MC_COS)
    int64_t n;              // database rows
    int64_t m;              // queries
    int kp;                 // padded K (multiple of 32)
    int kk;                 // candidates kept per query and split
    int splits;
    int64_t split_tiles;    // database tiles per split
    int64_t n_tiles;
    uint64_t *cand;
    int *err;
    // threshold-filter mode (candidate counts beyond the on-chip heaps): every
    // candidate with d~ <= thr[query] is appended to the query's list of fcap
    // keys; fcount[query] counts them all (also those past fcap)
    const float *thr;
    uint64_t *fout;
    int *fcount;
    int fcap;
    // locality order (allknn over a reordered database, heap mode only):
    // perm[p] = the 0-based id of the row at position p of the query and
    // database tiles; query CTA x starts its scan at database tile rot[x]
    // and wraps around.  Null: identity order, no rotation.
    const uint32_t *perm;
    const int *rot;
    // first query tile of this launch (a scan may be launched in waves of
    // query tiles, see launch_tc_scan)
    int64_t qt0;
    // heap mode: per-query bound shared by every heap of the query (all
    // splits and both column heaps), indexed by query position; null: none
    uint32_t *qbound;
};

template <int QT, int STAGES>
struct TcSmem {
    static size_t a_bytes(int kp) { return size_t(QT) * TILE * kp * 2; }
    static size_t b_bytes(int kp) { return size_t(STAGES) * TILE * kp * 2; }
    static size_t heap_bytes(int kk) { return size_t(QT) * TILE * col_splits<QT>() * (kk + kBufCap) * 8; }
    static size_t bar_bytes() { return 256; }
    static size_t total(int kp, int kk) { return 1024 + a_bytes(kp) + b_bytes(kp) + heap_bytes(kk) + bar_bytes(); }
};

// Epilogue warps of this CTA whose lane quarter holds at least one query: only
// they take part in the accumulator hand-off; the others leave at once.
template <int QT, int CS>
__device__ __forceinline__ int tc_live_warps(const TcArgs &a) {
    int live = 0;
    for (int q = 0; q < QT; ++q)
        for (int w = 0; w < 4; ++w)
            if ((a.qt0 + int64_t(blockIdx.x) * QT + q) * TILE + w * 32 < a.m) live += CS;
    return live;
}

// The scans' candidate handling of one 32-column chunk for one query row
// (one lane): the approximate distance of each column and the best per group
// of 8 columns, a warp vote on the chunk and on each group, then
//   heap mode: branch-free raw appends (the slot is always written with the
//     column's id and value, the count only advances for a candidate; the
//     key is made when the buffer drains into the lane's heap);
//   FILTER: every column at or below the query's fixed bound appended to
//     its list of fcap keys (fcount counts them all; rare, ~3 kk of n).
// DOT ranks by -v: its columns keep v, take the maximum and compare with
// -topd (exact: negation is exact).
template <int MC, bool FILTER = false>
struct ChunkTopK {
    uint64_t *heap, *cbuf;
    int hs, kk;
    int64_t n;
    const uint32_t *perm;
    bool qvalid;
    int nbuf;
    uint64_t top;
    float topd, ntopd;
    uint64_t *fout;  // FILTER: lists of fcap keys per query, counts
    int *fcount;
    int fcap;
    int64_t query;
    // the query's shared bound (heap mode): the filter threshold is the
    // smaller of this heap's frontier and the bound; a full heap lowers the
    // bound to its frontier
    uint32_t *qb;
    float bnd, published;

    __device__ __forceinline__ void set_threshold(float heap_frontier) {
        topd = !qvalid ? -INFINITY : fminf(heap_frontier, bnd);
        ntopd = -topd;
        if (qb && qvalid && heap_frontier < published) {
            bound_lower(qb, heap_frontier);
            published = heap_frontier;
        }
    }
    // once per database tile: pick up the bound the other heaps published
    __device__ __forceinline__ void refresh() {
        if (!qb || !qvalid) return;
        bnd = bound_read(qb);
        if (bnd < topd) { topd = bnd; ntopd = -bnd; }
    }

    __device__ __forceinline__ void chunk(const uint32_t (&r)[32], int64_t id0, const float *__restrict__ dnorm) {
        const float *nrm = dnorm + id0;
        float dv[32];
        float gbest[4];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const float v = __uint_as_float(r[j]);
            if (MC == MC_DOT) dv[j] = v;
            else if (MC == MC_SQ) dv[j] = fmaf(-2.0f, v, __ldg(nrm + j));
            else dv[j] = -v * __ldg(nrm + j);
        }
#pragma unroll
        for (int g = 0; g < 4; ++g) gbest[g] = MC == MC_DOT ? fmax8(dv + 8 * g) : fmin8(dv + 8 * g);
        const float cbest = MC == MC_DOT ? fmax3(fmax3(gbest[0], gbest[1], gbest[2]), gbest[3], gbest[3])
                                         : fmin3(fmin3(gbest[0], gbest[1], gbest[2]), gbest[3], gbest[3]);
        auto passes = [&](float x) { return MC == MC_DOT ? x >= ntopd : x <= topd; };
        if (!__any_sync(0xffffffffu, passes(cbest))) return;
        const int lim = int(id0 + 32 <= n ? 32 : n - id0);  // valid columns
        if constexpr (FILTER) {
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                if (passes(dv[j]) && j < lim && qvalid) {
                    const int pos = atomicAdd(fcount + query, 1);
                    if (pos < fcap)
                        fout[size_t(query) * fcap + pos] = make_key(MC == MC_DOT ? -dv[j] : dv[j], uint32_t(id0 + j));
                }
            }
        } else {
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                if (!__any_sync(0xffffffffu, passes(gbest[g]))) continue;
#pragma unroll
                for (int j = 8 * g; j < 8 * g + 8; ++j) {
                    cbuf[nbuf * hs] = (uint64_t(uint32_t(id0) + uint32_t(j)) << 32) | __float_as_uint(dv[j]);
                    nbuf += (passes(dv[j]) && j < lim) ? 1 : 0;
                }
                if (__any_sync(0xffffffffu, nbuf >= kDrainTrigger)) {
                    top = heap_drain_raw<MC == MC_DOT>(heap, cbuf, kk, hs, nbuf, top, perm);
                    nbuf = 0;
                    set_threshold(top == KEY_EMPTY ? INFINITY : key_dist(top));
                }
            }
        }
    }
};

template <int QT, int STAGES, int MC, bool FILTER>
__global__ void __launch_bounds__(tc_threads<QT>(), 1) tc_scan_kernel(TcArgs a) {
    constexpr int CS = col_splits<QT>();
    constexpr int NACC = acc_buffers<QT, FILTER>();
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // 1024-byte alignment for the swizzle atoms
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const size_t tile_bytes = size_t(TILE) * a.kp * 2;
    uint8_t *sA = smem;
    uint8_t *sB = sA + QT * tile_bytes;
    uint64_t *heap_base = reinterpret_cast<uint64_t *>(sB + STAGES * tile_bytes);
    uint64_t *buf_base = heap_base + size_t(QT) * TILE * CS * a.kk;
    uint64_t *bars = buf_base + size_t(QT) * TILE * CS * kBufCap;
    uint64_t *a_full = bars;
    uint64_t *full = bars + 1;
    uint64_t *empty = full + STAGES;
    uint64_t *acc_full = empty + STAGES;
    uint64_t *acc_empty = acc_full + NACC;
    uint64_t *mma_done = acc_empty + NACC;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);

    constexpr int NCOLS = QT * NACC * TILE;  // all 512 TMEM columns
    const int warp = threadIdx.x / 32;
    const int lane = threadIdx.x % 32;

    if (threadIdx.x == 0) {
        tc::mbar_init(a_full, 1);
        for (int s = 0; s < STAGES; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < NACC; ++b) {
            tc::mbar_init(&acc_full[b], 1);
            tc::mbar_init(&acc_empty[b], tc_live_warps<QT, CS>(a));
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
    // database tile of the CTA's t-th step: t_lo + t, rotated by rot[x]
    const int64_t rot = a.rot ? int64_t(a.rot[a.qt0 + blockIdx.x]) : 0;
    auto phys_tile = [&](int t) {
        int64_t p = t_lo + t + rot;
        return p >= a.n_tiles ? p - a.n_tiles : p;
    };

    if (warp == 0) {
        if (lane == 0) {
            tc::mbar_arrive_expect_tx(a_full, uint32_t(QT * tile_bytes));
            for (int q = 0; q < QT; ++q)
                tc::bulk_g2s(sA + q * tile_bytes, a.qt + (size_t(a.qt0) + size_t(blockIdx.x) * QT + q) * tile_bytes,
                             uint32_t(tile_bytes), a_full);
            int issued = 0;
            for (int t = 0; t < T_tiles; ++t) {
                const int s = t % STAGES;
                const uint32_t ph = (t / STAGES) & 1;
                if (!tc::mbar_wait(&empty[s], ph ^ 1, a.err, 1)) break;
                tc::mbar_arrive_expect_tx(&full[s], uint32_t(tile_bytes));
                tc::bulk_g2s(sB + s * tile_bytes, a.dt + size_t(phys_tile(t)) * tile_bytes, uint32_t(tile_bytes),
                             &full[s]);
                issued = t + 1;
            }
            // wait (bounded) until every copy this thread issued has landed
            tc::mbar_wait(a_full, 0, a.err, 2);
            for (int t = issued - STAGES < 0 ? 0 : issued - STAGES; t < issued; ++t)
                tc::mbar_wait(&full[t % STAGES], (t / STAGES) & 1, a.err, 2);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = tc::idesc_bf16_f32(TILE, TILE);
            bool ok = tc::mbar_wait(a_full, 0, a.err, 3);
            const uint32_t a_addr = tc::smem_u32(sA);
            const uint32_t b_addr0 = tc::smem_u32(sB);
            const int ksteps = a.kp / 16;
            int issued = 0;
            for (int t = 0; ok && t < T_tiles; ++t) {
                const int s = t % STAGES;
                const int b = t % NACC;
                if (!tc::mbar_wait(&full[s], (t / STAGES) & 1, a.err, 4)) break;
                if (!tc::mbar_wait(&acc_empty[b], ((t / NACC) & 1) ^ 1, a.err, 5)) break;
                tc::tc_fence_after();
                const uint32_t b_addr = b_addr0 + uint32_t(s * tile_bytes);
#pragma unroll
                for (int q = 0; q < QT; ++q) {
                    const uint32_t d_tmem = tmem_base + uint32_t((q * NACC + b) * TILE);
                    for (int kk = 0; kk < ksteps; ++kk) {
                        const uint32_t kbyte = uint32_t(kk) * 32u;
                        const uint32_t blk_off = (kbyte / SW) * (TILE * SW) + (kbyte % SW);
                        const uint64_t ad = tc::smem_desc(a_addr + uint32_t(q * tile_bytes) + blk_off, SW);
                        const uint64_t bd = tc::smem_desc(b_addr + blk_off, SW);
                        tc::mma_f16(d_tmem, ad, bd, idesc, kk > 0 ? 1u : 0u);
                    }
                }
                tc::mma_commit(&empty[s]);
                tc::mma_commit(&acc_full[b]);
                issued = t + 1;
            }
            (void)issued;
            tc::mma_commit(mma_done);
            tc::mbar_wait(mma_done, 0, a.err, 6);
        }
        __syncwarp();
    } else {
        const int e = warp - 2;
        const int q = e / (4 * CS);
        const int cs = (e / 4) % CS;
        const int quarter = warp % 4;
        const int row = quarter * 32 + lane;
        const int64_t query = (a.qt0 + int64_t(blockIdx.x) * QT + q) * TILE + row;
        constexpr int hs = QT * TILE * CS;
        constexpr int CHUNKS = TILE / 32 / CS;  // 32-column chunks per warp and tile
        // padding rows of a partial query tile filter everything out (a
        // -inf threshold), and warps holding only padding rows skip the
        // epilogue: they just hand the accumulator back
        ChunkTopK<MC, FILTER> T;
        T.heap = heap_base + (e * 32 + lane);
        T.cbuf = buf_base + (e * 32 + lane);
        T.hs = hs;
        T.kk = a.kk;
        T.n = a.n;
        T.perm = a.perm;
        T.qvalid = query < a.m;
        T.nbuf = 0;
        T.top = KEY_EMPTY;
        T.topd = T.qvalid ? (FILTER ? a.thr[query] : INFINITY) : -INFINITY;
        T.ntopd = -T.topd;
        T.fout = a.fout;
        T.fcount = a.fcount;
        T.fcap = a.fcap;
        T.query = query;
        T.qb = (!FILTER && a.qbound && T.qvalid) ? a.qbound + query : nullptr;
        T.bnd = INFINITY;
        T.published = INFINITY;
        if (!FILTER) Heap{T.heap, a.kk, hs}.init();
        const bool warp_live = (a.qt0 + int64_t(blockIdx.x) * QT + q) * TILE + quarter * 32 < a.m;
        for (int t = 0; warp_live && t < T_tiles; ++t) {
            const int b = t % NACC;
            int ok = 1;
            if (lane == 0) ok = tc::mbar_wait(&acc_full[b], (t / NACC) & 1, a.err, 7) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) break;
            tc::tc_fence_after();
            T.refresh();
            const int64_t row0 = phys_tile(t) * TILE + cs * (TILE / CS);
            // this warp's columns in flight together, one wait, then the
            // accumulator goes back to the MMA warp before any filtering
            uint32_t r[CHUNKS][32];
            __syncwarp();
            const uint32_t tbase = tmem_base + (uint32_t(quarter * 32) << 16) +
                                   uint32_t((q * NACC + b) * TILE + cs * (TILE / CS));
#pragma unroll
            for (int c = 0; c < CHUNKS; ++c) tc::tmem_ld_32x32b_x32_async(tbase + uint32_t(c * 32), r[c]);
            tc::tmem_wait_ld();
            tc::tc_fence_before();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&acc_empty[b]);
#pragma unroll
            for (int c = 0; c < CHUNKS; ++c) T.chunk(r[c], row0 + c * 32, a.dnorm);
        }
        if (!FILTER) T.top = heap_drain_raw<MC == MC_DOT>(T.heap, T.cbuf, a.kk, hs, T.nbuf, T.top, a.perm);
        Heap H{T.heap, a.kk, hs};
        if (!FILTER && query < a.m) {
            H.sort_ascending();
            // the candidates of a query go to its row by id
            const size_t qrow = a.perm ? size_t(a.perm[query]) : size_t(query);
            uint64_t *out = a.cand + ((qrow * a.splits + blockIdx.y) * CS + cs) * a.kk;
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

template <int QT, int STAGES, int MC, bool FILTER>
cudaError_t launch_tc_t(const TcArgs &a, cudaStream_t st) {
    size_t smem = TcSmem<QT, STAGES>::total(a.kp, a.kk);
    if (acc_buffers<QT, FILTER>() * QT * TILE == 512 && smem < kAloneSmem) smem = kAloneSmem;
    auto kern = tc_scan_kernel<QT, STAGES, MC, FILTER>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    dim3 grid(unsigned((a.m + QT * TILE - 1) / (QT * TILE)), unsigned(a.splits));
    TcArgs b = a;
    b.qt0 = 0;
    kern<<<grid, tc_threads<QT>(), smem, st>>>(b);
    return cudaGetLastError();
}

template <int QT, int STAGES, bool FILTER = false>
cudaError_t launch_tc_mc(const TcArgs &a, int mc, cudaStream_t st) {
    if (mc == MC_SQ) return launch_tc_t<QT, STAGES, MC_SQ, FILTER>(a, st);
    if (mc == MC_COS) return launch_tc_t<QT, STAGES, MC_COS, FILTER>(a, st);
    return launch_tc_t<QT, STAGES, MC_DOT, FILTER>(a, st);
}

// ---------------------------------------------------------------------------
// The wide scan: 256 database rows per MMA (M = 128 queries x N = 256).
//
// A 128 x 128 x 16 tcgen05.mma occupies the tensor pipe for 64 cycles, and
// every MMA and commit adds a fixed cost, so a 128 x 128 tile of 6 MMAs + 2
// commits runs at ~80% of the pipe's rate even with nothing else on the SM;
// at N = 256 each MMA is 128 cycles and the commits hide behind it.  The
// database streams through a ring of K-blocks (256 rows x 32 BF16, the two
// 128-row tiles' K-blocks side by side: 16 KB), so the heaps still fit next
// to the ring.  Two accumulators of 128 x 256 FP32 fill all 512 TMEM
// columns.  Roles, heaps, outputs and the locality order are those of
// tc_scan_kernel (one query tile per CTA, two epilogue warps per TMEM lane
// quarter, each owning alternate 32-column chunks and its own heap).
// ---------------------------------------------------------------------------
constexpr int WIDE = 2 * TILE;          // database rows per wide tile
constexpr int KBLK = TILE * SW;         // bytes of one K-block of a 128-row tile

template <int KST>
struct WideSmem {
    static size_t total(int kp, int kk) {
        return 1024 + size_t(TILE) * kp * 2 + size_t(KST) * 2 * KBLK + TcSmem<1, 1>::heap_bytes(kk) + 256;
    }
};

template <int KST, int MC>
__global__ void __launch_bounds__(tc_threads<1>(), 1) tc_wide_kernel(TcArgs a) {
    constexpr int CS = 2;
    constexpr int NACC = 2;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const size_t tile_bytes = size_t(TILE) * a.kp * 2;  // one 128-row tile (all K-blocks)
    const int kblocks = a.kp / KBE;
    uint8_t *sA = smem;
    uint8_t *sB = sA + tile_bytes;  // KST stages of 2 x KBLK bytes
    uint64_t *heap_base = reinterpret_cast<uint64_t *>(sB + size_t(KST) * 2 * KBLK);
    uint64_t *buf_base = heap_base + size_t(TILE) * CS * a.kk;
    uint64_t *bars = buf_base + size_t(TILE) * CS * kBufCap;
    uint64_t *a_full = bars;
    uint64_t *full = bars + 1;
    uint64_t *empty = full + KST;
    uint64_t *acc_full = empty + KST;
    uint64_t *acc_empty = acc_full + NACC;
    uint64_t *mma_done = acc_empty + NACC;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);
    const int warp = threadIdx.x / 32;
    const int lane = threadIdx.x % 32;

    if (threadIdx.x == 0) {
        tc::mbar_init(a_full, 1);
        for (int s = 0; s < KST; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < NACC; ++b) {
            tc::mbar_init(&acc_full[b], 1);
            tc::mbar_init(&acc_empty[b], tc_live_warps<1, CS>(a));
        }
        tc::mbar_init(mma_done, 1);
        tc::fence_mbarrier_init();
    }
    if (warp == 1) tc::tmem_alloc<512>(tmem_slot);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    // wide tiles (pairs of 128-row tiles: the tile set holds an even count);
    // split ranges and the locality rotation in wide tiles
    const int64_t n_wide = (a.n_tiles + 1) / 2;
    const int64_t split_w = (n_wide + a.splits - 1) / a.splits;
    const int64_t w_lo = int64_t(blockIdx.y) * split_w;
    const int64_t w_hi = w_lo + split_w < n_wide ? w_lo + split_w : n_wide;
    const int W = w_hi > w_lo ? int(w_hi - w_lo) : 0;
    const int64_t qx = a.qt0 + blockIdx.x;  // query tile
    const int64_t rot = a.rot ? int64_t(a.rot[qx]) / 2 : 0;
    auto phys_wide = [&](int u) {
        int64_t p = w_lo + u + rot;
        return p >= n_wide ? p - n_wide : p;
    };

    if (warp == 0) {
        if (lane == 0) {
            tc::mbar_arrive_expect_tx(a_full, uint32_t(tile_bytes));
            tc::bulk_g2s(sA, a.qt + size_t(qx) * tile_bytes, uint32_t(tile_bytes), a_full);
            const int steps = W * kblocks;
            int issued = 0;
            for (int st = 0; st < steps; ++st) {
                const int s = st % KST;
                if (!tc::mbar_wait(&empty[s], ((st / KST) & 1) ^ 1, a.err, 1)) break;
                const int u = st / kblocks, kb = st % kblocks;
                const uint8_t *src = a.dt + size_t(2 * phys_wide(u)) * tile_bytes + size_t(kb) * KBLK;
                uint8_t *dst = sB + size_t(s) * 2 * KBLK;
                tc::mbar_arrive_expect_tx(&full[s], uint32_t(2 * KBLK));
                tc::bulk_g2s(dst, src, uint32_t(KBLK), &full[s]);
                tc::bulk_g2s(dst + KBLK, src + tile_bytes, uint32_t(KBLK), &full[s]);
                issued = st + 1;
            }
            // wait (bounded) until every copy this thread issued has landed
            tc::mbar_wait(a_full, 0, a.err, 2);
            for (int st = issued - KST < 0 ? 0 : issued - KST; st < issued; ++st)
                tc::mbar_wait(&full[st % KST], (st / KST) & 1, a.err, 2);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = tc::idesc_bf16_f32(TILE, WIDE);
            bool ok = tc::mbar_wait(a_full, 0, a.err, 3);
            const uint32_t a_addr = tc::smem_u32(sA);
            const uint32_t b_addr0 = tc::smem_u32(sB);
            for (int u = 0; ok && u < W; ++u) {
                const int b = u & 1;
                if (!tc::mbar_wait(&acc_empty[b], ((u >> 1) & 1) ^ 1, a.err, 5)) break;
                const uint32_t d_tmem = tmem_base + uint32_t(b * WIDE);
                for (int kb = 0; ok && kb < kblocks; ++kb) {
                    const int st = u * kblocks + kb;
                    const int s = st % KST;
                    if (!tc::mbar_wait(&full[s], (st / KST) & 1, a.err, 4)) { ok = false; break; }
                    tc::tc_fence_after();
#pragma unroll
                    for (int h = 0; h < 2; ++h) {  // two K = 16 steps per 32-element K-block
                        const uint64_t ad = tc::smem_desc(a_addr + uint32_t(kb * KBLK + h * 32), SW);
                        const uint64_t bd = tc::smem_desc(b_addr0 + uint32_t(s * 2 * KBLK + h * 32), SW);
                        tc::mma_f16(d_tmem, ad, bd, idesc, (kb > 0 || h > 0) ? 1u : 0u);
                    }
                    tc::mma_commit(&empty[s]);
                }
                if (!ok) break;
                tc::mma_commit(&acc_full[b]);
            }
            tc::mma_commit(mma_done);
            tc::mbar_wait(mma_done, 0, a.err, 6);
        }
        __syncwarp();
    } else {
        const int e = warp - 2;
        const int cs = e / 4;
        const int quarter = warp % 4;
        const int row = quarter * 32 + lane;
        const int64_t query = qx * TILE + row;
        constexpr int hs = TILE * CS;
        ChunkTopK<MC> T;
        T.heap = heap_base + (e * 32 + lane);
        T.cbuf = buf_base + (e * 32 + lane);
        T.hs = hs;
        T.kk = a.kk;
        T.n = a.n;
        T.perm = a.perm;
        T.qvalid = query < a.m;
        T.nbuf = 0;
        T.top = KEY_EMPTY;
        T.topd = T.qvalid ? INFINITY : -INFINITY;
        T.ntopd = -T.topd;
        T.fout = nullptr;
        T.fcount = nullptr;
        T.fcap = 0;
        T.query = query;
        T.qb = (a.qbound && T.qvalid) ? a.qbound + query : nullptr;
        T.bnd = INFINITY;
        T.published = INFINITY;
        Heap{T.heap, a.kk, hs}.init();
        const bool warp_live = qx * TILE + quarter * 32 < a.m;
        for (int u = 0; warp_live && u < W; ++u) {
            const int b = u & 1;
            int ok = 1;
            if (lane == 0) ok = tc::mbar_wait(&acc_full[b], (u >> 1) & 1, a.err, 7) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) break;
            tc::tc_fence_after();
            T.refresh();
            // this warp's 128 columns: the 32-column chunks cs, cs + 2, ...
            // of the wide tile, so that a group of neighbouring rows in the
            // locality order feeds both heaps of a query evenly.  LDC
            // 32-column loads in flight per round; the accumulator goes back
            // to the MMA warp as soon as the last load landed (two
            // accumulators only: the MMAs must not wait for the filtering).
            // DOT holds all four chunks in registers; the norm-scaled metrics
            // need registers for the distances and take two rounds of two.
            constexpr int LDC = MC == MC_DOT ? 4 : 2;
            const int64_t row0 = phys_wide(u) * WIDE + cs * 32;
            const uint32_t tbase = tmem_base + (uint32_t(quarter * 32) << 16) + uint32_t(b * WIDE + cs * 32);
            uint32_t r[LDC][32];
#pragma unroll
            for (int round = 0; round < 4 / LDC; ++round) {
                __syncwarp();
#pragma unroll
                for (int c = 0; c < LDC; ++c)
                    tc::tmem_ld_32x32b_x32_async(tbase + uint32_t((round * LDC + c) * 64), r[c]);
                tc::tmem_wait_ld();
                if (round == 4 / LDC - 1) {
                    tc::tc_fence_before();
                    __syncwarp();
                    if (lane == 0) tc::mbar_arrive(&acc_empty[b]);
                }
#pragma unroll
                for (int c = 0; c < LDC; ++c) T.chunk(r[c], row0 + (round * LDC + c) * 64, a.dnorm);
            }
        }
        T.top = heap_drain_raw<MC == MC_DOT>(T.heap, T.cbuf, a.kk, hs, T.nbuf, T.top, a.perm);
        if (query < a.m) {
            Heap H{T.heap, a.kk, hs};
            H.sort_ascending();
            const size_t qrow = a.perm ? size_t(a.perm[query]) : size_t(query);
            uint64_t *out = a.cand + ((qrow * a.splits + blockIdx.y) * CS + cs) * a.kk;
            for (int i = 0; i < a.kk; ++i) out[i] = H.h[i * hs];
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc::tc_fence_after();
        tc::tmem_dealloc<512>(tmem_base);
    }
}

// Launches the wide scan over all query tiles, `wave` query tiles per
// launch (0: one launch).  A wave of one CTA per SM starts together, so with
// the locality order (query tile x starting at database tile ~x) its CTAs
// read a sliding window of neighbouring database tiles at any moment and the
// database streams through L2 about once per wave; one launch of every tile
// instead staggers the CTAs' start times over the whole scan.
template <int KST, int MC>
cudaError_t launch_wide_t(const TcArgs &a, cudaStream_t st, int64_t wave, int *launches) {
    size_t smem = WideSmem<KST>::total(a.kp, a.kk);
    if (smem < kAloneSmem) smem = kAloneSmem;  // all 512 TMEM columns: alone on the SM
    auto kern = tc_wide_kernel<KST, MC>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    const int64_t qtiles = (a.m + TILE - 1) / TILE;
    const int64_t per = wave > 0 ? wave : qtiles;
    for (int64_t t0 = 0; t0 < qtiles; t0 += per) {
        TcArgs b = a;
        b.qt0 = t0;
        dim3 grid(unsigned(std::min<int64_t>(per, qtiles - t0)), unsigned(a.splits));
        kern<<<grid, tc_threads<1>(), smem, st>>>(b);
        if (launches) *launches += 1;
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <int KST>
cudaError_t launch_wide_mc(const TcArgs &a, int mc, cudaStream_t st, int64_t wave, int *launches) {
    if (mc == MC_SQ) return launch_wide_t<KST, MC_SQ>(a, st, wave, launches);
    if (mc == MC_COS) return launch_wide_t<KST, MC_COS>(a, st, wave, launches);
    return launch_wide_t<KST, MC_DOT>(a, st, wave, launches);
}

// The database tiles seen by the tensor-map TMA as a 2D array of 64-byte
// lines (32 BF16, already swizzled): line (tile * kblocks + kb) * 128 + r is
// row r of K-block kb of a tile, so one 32 x 128 box is one tile's K-block,
// copied verbatim (no swizzle mode: the bytes already are in the MMA's
// layout).  The tile set holds an even number of tiles.
cudaError_t database_line_map(const TcArgs &a, CUtensorMap *map) {
    using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static EncodeFn encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return e;
        if (q != cudaDriverEntryPointSuccess || !fn) return cudaErrorNotSupported;
        encode = reinterpret_cast<EncodeFn>(fn);
    }
    if (reinterpret_cast<uintptr_t>(a.dt) % 16 != 0) return cudaErrorInvalidValue;
    const cuuint64_t lines = cuuint64_t((a.n_tiles + 1) / 2 * 2) * cuuint64_t(a.kp / KBE) * TILE;
    const cuuint64_t dims[2] = {cuuint64_t(KBE), lines};
    const cuuint64_t strides[1] = {cuuint64_t(SW)};
    const cuuint32_t box[2] = {cuuint32_t(KBE), cuuint32_t(TILE)};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<uint8_t *>(a.dt), dims, strides, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// The pair scan: the wide scan on CTA pairs (clusters of two) with M = 256
// MMAs (tcgen05 cta_group::2).  Each CTA owns one 128-row query tile, as in
// the wide scan, and both CTAs of a pair scan the same database tiles; the
// even CTA issues one 256 x 256 x 16 MMA per K step that reads the query
// tiles of both CTAs and the database rows of both: rows 0..127 of each
// 256-row wide tile sit in the even CTA's ring, rows 128..255 in the odd
// one's.  So each SM loads half of every database K-block (8 KB instead of
// 16 KB): half the L2 -> SM traffic per query, and a ring twice as deep in
// the same shared memory to cover the copies' latency.  Each CTA's TMEM
// holds its own 128 query rows x 256 columns, so the epilogue is the wide
// scan's.
//
// Hand-offs.  Each CTA's copies complete on its own mbarriers.  The odd
// CTA's warp 1 forwards every landed copy (its query tile, each ring stage)
// to an mbarrier in the even CTA (pa_full, pfull[s]), where the MMA thread
// waits for both halves.  The MMA thread's commits arrive on the barriers of
// both CTAs (empty[s] for the producers, acc_full[b] for the epilogues).
// The odd CTA's epilogue warps release an accumulator by arriving on the
// even CTA's pacc_empty[b].  Every wait is bounded; both CTAs meet at a
// cluster barrier before TMEM is freed, so no CTA leaves while the other's
// MMAs may still read its shared memory.
// ---------------------------------------------------------------------------
constexpr int PKBLK = TILE * SW;  // one 128-row half of a wide K-block: 8 KB

template <int KST, int CS = 2>
struct PairSmem {
    static size_t total(int kp, int kk) {
        return 1024 + size_t(TILE) * kp * 2 + size_t(KST) * PKBLK + size_t(TILE) * CS * (kk + kBufCap) * 8 + 512;
    }
};

// CS heaps per query: 2 (two epilogue warps per TMEM lane quarter, each
// filtering one 128-column half of every wide tile into its own heap), or 1
// (one warp per quarter filtering both halves into one heap: half the heap
// memory, for candidate lists twice as long).
template <int KST, int MC, int CS>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(64 + TILE * CS, 1)
    tc_pair_kernel(TcArgs a, const __grid_constant__ CUtensorMap dmap) {
    constexpr int NACC = 2;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const size_t tile_bytes = size_t(TILE) * a.kp * 2;
    const int kblocks = a.kp / KBE;
    uint8_t *sA = smem;
    uint8_t *sB = sA + tile_bytes;  // KST stages of PKBLK bytes
    uint64_t *heap_base = reinterpret_cast<uint64_t *>(sB + size_t(KST) * PKBLK);
    uint64_t *buf_base = heap_base + size_t(TILE) * CS * a.kk;
    uint64_t *bars = buf_base + size_t(TILE) * CS * kBufCap;
    uint64_t *a_full = bars;                 // this CTA's query tile landed
    uint64_t *pa_full = a_full + 1;          // (even CTA) the odd CTA's query tile landed
    uint64_t *full = pa_full + 1;            // (even CTA) both halves of stage s landed
    uint64_t *empty = full + KST;            // the MMAs of stage s are done
    uint64_t *acc_full = empty + KST;        // accumulator b holds a finished wide tile
    uint64_t *acc_empty = acc_full + NACC;   // (even CTA) its epilogue warps released b
    uint64_t *pacc_empty = acc_empty + NACC; // (even CTA) the odd CTA's epilogue warps released b
    uint64_t *mma_done = pacc_empty + NACC;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);
    const int warp = threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    const uint32_t rank = tc::cluster_ctarank();  // 0: the even CTA (issues the MMAs)
    const uint32_t peer = rank ^ 1u;
    const int64_t qx = a.qt0 + blockIdx.x;  // this CTA's query tile
    const int64_t qpair = qx - int64_t(rank);
    // live epilogue warps of a query tile: its lane quarters holding a query
    auto live_warps = [&](int64_t tile) {
        int live = 0;
        for (int w = 0; w < 4; ++w)
            if (tile * TILE + w * 32 < a.m) live += CS;
        return live;
    };
    const int live_self = live_warps(qx), live_peer = live_warps(qpair + int64_t(peer));

    if (threadIdx.x == 0) {
        tc::mbar_init(a_full, 1);
        tc::mbar_init(pa_full, 1);
        for (int s = 0; s < KST; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < NACC; ++b) {
            tc::mbar_init(&acc_full[b], 1);
            tc::mbar_init(&acc_empty[b], live_self > 0 ? live_self : 1);
            tc::mbar_init(&pacc_empty[b], live_peer > 0 ? live_peer : 1);
        }
        tc::mbar_init(mma_done, 1);
        tc::fence_mbarrier_init();
    }
    if (warp == 1) tc::tmem_alloc_pair<512>(tmem_slot);
    tc::tc_fence_before();
    __syncthreads();
    tc::cluster_sync();  // both CTAs' barriers exist before any cross-CTA arrive
    tc::tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    // wide tiles and the scan order: both CTAs of a pair follow the even
    // CTA's query tile's locality rotation
    const int64_t n_wide = (a.n_tiles + 1) / 2;
    const int64_t split_w = (n_wide + a.splits - 1) / a.splits;
    const int64_t w_lo = int64_t(blockIdx.y) * split_w;
    const int64_t w_hi = w_lo + split_w < n_wide ? w_lo + split_w : n_wide;
    const int W = w_hi > w_lo ? int(w_hi - w_lo) : 0;
    const int64_t rot = a.rot ? int64_t(a.rot[qpair]) / 2 : 0;
    auto phys_wide = [&](int u) {
        int64_t p = w_lo + u + rot;
        return p >= n_wide ? p - n_wide : p;
    };
    const int steps = W * kblocks;

    if (warp == 0) {
        if (lane == 0) {
            // producer: this CTA's query tile, then its half of every K-block.
            // Both halves of stage s complete on the even CTA's full[s]: the
            // even CTA arms it for both, the odd CTA's TMA counts its bytes
            // there directly (cta_group::2), so no thread relays them.
            tc::mbar_arrive_expect_tx(a_full, uint32_t(tile_bytes));
            tc::bulk_g2s(sA, a.qt + size_t(qx) * tile_bytes, uint32_t(tile_bytes), a_full);
            const uint32_t full0 = tc::mapa_shared(tc::smem_u32(full), 0);
            int issued = 0;
            for (int st = 0; st < steps; ++st) {
                const int s = st % KST;
                if (!tc::mbar_wait(&empty[s], ((st / KST) & 1) ^ 1, a.err, 1)) break;
                const int u = st / kblocks, kb = st % kblocks;
                const int64_t tile = 2 * phys_wide(u) + rank;
                if (rank == 0) {
                    tc::mbar_arrive_expect_tx(&full[s], uint32_t(2 * PKBLK));
                    tc::bulk_g2s(sB + size_t(s) * PKBLK, a.dt + size_t(tile) * tile_bytes + size_t(kb) * KBLK,
                                 uint32_t(PKBLK), &full[s]);
                } else {
                    tc::tma_load_2d_pair(sB + size_t(s) * PKBLK, &dmap, 0, int((tile * kblocks + kb) * TILE),
                                         full0 + uint32_t(s * 8));
                }
                issued = st + 1;
            }
            // wait (bounded) until every copy of this CTA pair has landed
            // (the even CTA's barriers count both halves; the final cluster
            // barrier keeps the odd CTA alive until then)
            tc::mbar_wait(a_full, 0, a.err, 2);
            if (rank == 0)
                for (int st = issued - KST < 0 ? 0 : issued - KST; st < issued; ++st)
                    tc::mbar_wait(&full[st % KST], (st / KST) & 1, a.err, 2);
        }
    } else if (warp == 1) {
        if (lane == 0 && rank == 1) {
            // the odd CTA tells the even CTA that its query tile landed
            if (tc::mbar_wait(a_full, 0, a.err, 8)) tc::mbar_arrive_cluster(tc::mapa_shared(tc::smem_u32(pa_full), peer));
        } else if (lane == 0) {
            // the even CTA issues the pair MMAs
            constexpr uint32_t idesc = tc::idesc_bf16_f32(2 * TILE, WIDE);
            bool ok = tc::mbar_wait(a_full, 0, a.err, 3) && tc::mbar_wait(pa_full, 0, a.err, 3);
            const uint32_t a_addr = tc::smem_u32(sA);
            const uint32_t b_addr0 = tc::smem_u32(sB);
            const uint32_t r_empty0 = tc::mapa_shared(tc::smem_u32(empty), peer);
            const uint32_t r_acc_full0 = tc::mapa_shared(tc::smem_u32(acc_full), peer);
            for (int u = 0; ok && u < W; ++u) {
                const int b = u & 1;
                const uint32_t ph = ((u >> 1) & 1) ^ 1;
                if (!tc::mbar_wait(&acc_empty[b], ph, a.err, 5)) break;
                if (live_peer > 0 && !tc::mbar_wait(&pacc_empty[b], ph, a.err, 5)) break;
                const uint32_t d_tmem = tmem_base + uint32_t(b * WIDE);
                for (int kb = 0; ok && kb < kblocks; ++kb) {
                    const int st = u * kblocks + kb;
                    const int s = st % KST;
                    if (!tc::mbar_wait(&full[s], (st / KST) & 1, a.err, 4)) { ok = false; break; }
                    tc::tc_fence_after();
#pragma unroll
                    for (int h = 0; h < 2; ++h) {  // two K = 16 steps per 32-element K-block
                        const uint64_t ad = tc::smem_desc(a_addr + uint32_t(kb * KBLK + h * 32), SW);
                        const uint64_t bd = tc::smem_desc(b_addr0 + uint32_t(s * PKBLK + h * 32), SW);
                        tc::mma_f16_pair(d_tmem, ad, bd, idesc, (kb > 0 || h > 0) ? 1u : 0u);
                    }
                    tc::mma_commit_pair(tc::smem_u32(&empty[s]));
                    tc::mma_commit_pair(r_empty0 + uint32_t(s * 8));
                }
                if (!ok) break;
                tc::mma_commit_pair(tc::smem_u32(&acc_full[b]));
                tc::mma_commit_pair(r_acc_full0 + uint32_t(b * 8));
            }
            tc::mma_commit_pair(tc::smem_u32(mma_done));
            tc::mbar_wait(mma_done, 0, a.err, 6);
        }
        __syncwarp();
    } else {
        const int e = warp - 2;
        const int cs = e / 4;
        const int quarter = warp % 4;
        const int row = quarter * 32 + lane;
        const int64_t query = qx * TILE + row;
        constexpr int hs = TILE * CS;
        const uint32_t r_pacc0 = tc::mapa_shared(tc::smem_u32(pacc_empty), peer);
        ChunkTopK<MC> T;
        T.heap = heap_base + (e * 32 + lane);
        T.cbuf = buf_base + (e * 32 + lane);
        T.hs = hs;
        T.kk = a.kk;
        T.n = a.n;
        T.perm = a.perm;
        T.qvalid = query < a.m;
        T.nbuf = 0;
        T.top = KEY_EMPTY;
        T.topd = T.qvalid ? INFINITY : -INFINITY;
        T.ntopd = -T.topd;
        T.fout = nullptr;
        T.fcount = nullptr;
        T.fcap = 0;
        T.query = query;
        T.qb = (a.qbound && T.qvalid) ? a.qbound + query : nullptr;
        T.bnd = INFINITY;
        T.published = INFINITY;
        Heap{T.heap, a.kk, hs}.init();
        const bool warp_live = qx * TILE + quarter * 32 < a.m;
        for (int u = 0; warp_live && u < W; ++u) {
            const int b = u & 1;
            int ok = 1;
            if (lane == 0) ok = tc::mbar_wait(&acc_full[b], (u >> 1) & 1, a.err, 7) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) break;
            tc::tc_fence_after();
            T.refresh();
            constexpr int LDC = MC == MC_DOT ? 4 : 2;
            uint32_t r[LDC][32];
            // this warp's halves of the wide tile, each the 32-column chunks
            // half, half + 2, ... (one half with two heaps per query, so that
            // a group of neighbouring rows feeds both heaps evenly; both
            // with one); the accumulator goes back after the last load of
            // the last half
#pragma unroll
            for (int hc = 0; hc < 2 / CS; ++hc) {
                const int half = cs + hc;
                const int64_t row0 = phys_wide(u) * WIDE + half * 32;
                const uint32_t tbase = tmem_base + (uint32_t(quarter * 32) << 16) + uint32_t(b * WIDE + half * 32);
#pragma unroll
                for (int round = 0; round < 4 / LDC; ++round) {
                    __syncwarp();
#pragma unroll
                    for (int c = 0; c < LDC; ++c)
                        tc::tmem_ld_32x32b_x32_async(tbase + uint32_t((round * LDC + c) * 64), r[c]);
                    tc::tmem_wait_ld();
                    if (hc == 2 / CS - 1 && round == 4 / LDC - 1) {
                        tc::tc_fence_before();
                        __syncwarp();
                        if (lane == 0) {
                            if (rank == 0) tc::mbar_arrive(&acc_empty[b]);
                            else tc::mbar_arrive_cluster(r_pacc0 + uint32_t(b * 8));
                        }
                    }
#pragma unroll
                    for (int c = 0; c < LDC; ++c) T.chunk(r[c], row0 + (round * LDC + c) * 64, a.dnorm);
                }
            }
        }
        T.top = heap_drain_raw<MC == MC_DOT>(T.heap, T.cbuf, a.kk, hs, T.nbuf, T.top, a.perm);
        if (query < a.m) {
            Heap H{T.heap, a.kk, hs};
            H.sort_ascending();
            const size_t qrow = a.perm ? size_t(a.perm[query]) : size_t(query);
            uint64_t *out = a.cand + ((qrow * a.splits + blockIdx.y) * CS + cs) * a.kk;
            for (int i = 0; i < a.kk; ++i) out[i] = H.h[i * hs];
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::cluster_sync();  // the even CTA's MMAs are done with both CTAs' shared memory
    if (warp == 1) {
        tc::tc_fence_after();
        tc::tmem_dealloc_pair<512>(tmem_base);
    }
}

// Launches the pair scan over all query tiles (rounded up to an even count:
// the query tile sets are allocated in pairs), `wave` query tiles per launch
// (0: one launch; rounded up to an even count).
template <int KST, int MC, int CS>
cudaError_t launch_pair_t(const TcArgs &a, cudaStream_t st, int64_t wave, int *launches) {
    size_t smem = PairSmem<KST, CS>::total(a.kp, a.kk);
    if (smem < kAloneSmem) smem = kAloneSmem;  // all 512 TMEM columns: alone on the SM
    auto kern = tc_pair_kernel<KST, MC, CS>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    CUtensorMap dmap;
    e = database_line_map(a, &dmap);
    if (e != cudaSuccess) return e;
    const int64_t qtiles = ((a.m + TILE - 1) / TILE + 1) / 2 * 2;
    const int64_t per = wave > 0 ? (wave + 1) / 2 * 2 : qtiles;
    for (int64_t t0 = 0; t0 < qtiles; t0 += per) {
        TcArgs b = a;
        b.qt0 = t0;
        dim3 grid(unsigned(std::min<int64_t>(per, qtiles - t0)), unsigned(a.splits));
        kern<<<grid, 64 + TILE * CS, smem, st>>>(b, dmap);
        if (launches) *launches += 1;
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <int KST, int CS = 2>
cudaError_t launch_pair_mc(const TcArgs &a, int mc, cudaStream_t st, int64_t wave, int *launches) {
    if (mc == MC_SQ) return launch_pair_t<KST, MC_SQ, CS>(a, st, wave, launches);
    if (mc == MC_COS) return launch_pair_t<KST, MC_COS, CS>(a, st, wave, launches);
    return launch_pair_t<KST, MC_DOT, CS>(a, st, wave, launches);
}

// thr[q] = the smallest over the query's segments of the segment's last
// (kk-th) key distance: a bound with at least kk sample candidates below it.
__global__ void sample_bound_kernel(const uint64_t *__restrict__ cand, int64_t m, int segs, int kk,
                                    float *__restrict__ thr) {
    const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (q >= m) return;
    float b = INFINITY;
    for (int s = 0; s < segs; ++s) {
        const uint64_t key = cand[(size_t(q) * segs + s) * kk + kk - 1];
        if (key != KEY_EMPTY) b = fminf(b, key_dist(key));
    }
    thr[q] = b;
}

// Per query: sorts the filtered keys and keeps the first kk (sorted); a query
// whose list holds fewer than kk keys or overflowed is flagged for the exact
// fallback (its row is filled with empty keys).
__global__ void filter_select_kernel(const uint64_t *__restrict__ fout, const int *__restrict__ fcount, int fcap,
                                     int kk, uint64_t *__restrict__ cand, int *__restrict__ flags,
                                     int *__restrict__ flag_count) {
    extern __shared__ uint64_t sk[];
    const int64_t q = blockIdx.x;
    const int cnt = fcount[q];
    uint64_t *out = cand + size_t(q) * kk;
    if (cnt < kk || cnt > fcap) {
        for (int i = threadIdx.x; i < kk; i += blockDim.x) out[i] = KEY_EMPTY;
        if (threadIdx.x == 0) {
            flags[q] = 1;
            atomicAdd(flag_count, 1);
        }
        return;
    }
    int P = 1;
    while (P < cnt) P <<= 1;
    const uint64_t *src = fout + size_t(q) * fcap;
    for (int i = threadIdx.x; i < P; i += blockDim.x) sk[i] = i < cnt ? src[i] : KEY_EMPTY;
    block_bitonic_sort(sk, P);
    for (int i = threadIdx.x; i < kk; i += blockDim.x) out[i] = sk[i];
}

// ---------------------------------------------------------------------------
// Locality order for allknn.  Rows are grouped by their nearest pivot (P
// evenly spaced database rows) and the groups follow the pivots' chain
// order (pivots near each other in nearby places), so a query tile's near
// neighbours sit in its own group and the few after it, and each query CTA
// starts its scan at its group.  The heaps then hold close
// candidates after a few tiles and later tiles rarely pass the frontier: far
// fewer heap insertions than in id order, where the frontier only tightens
// as ~kk * ln(columns seen).  The kept (distance, id) keys, and so the
// results, do not depend on the order.
// ---------------------------------------------------------------------------
// pivot[i] = bucket of row i: the chain place rank[p] (or p itself, rank
// null) of its best pivot p among its segment keys (a kk = 1 scan of the
// rows against the pivots); count[bucket] += 1
__global__ void nearest_pivot_kernel(const uint64_t *__restrict__ cand, int64_t n, int segs,
                                     const uint32_t *__restrict__ rank, uint32_t *__restrict__ pivot,
                                     int *__restrict__ count) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t best = KEY_EMPTY;
    for (int s = 0; s < segs; ++s) best = min(best, cand[size_t(i) * segs + s]);
    uint32_t p = best == KEY_EMPTY ? 0u : key_id0(best);
    if (rank) p = rank[p];
    pivot[i] = p;
    atomicAdd(count + p, 1);
}

// start[b] = first position of bucket b (exclusive prefix sum of count), one
// block; cursor = a copy for the scatter
__global__ void bucket_offsets_kernel(const int *__restrict__ count, int P, int *__restrict__ start,
                                      int *__restrict__ cursor) {
    __shared__ int part[1024];
    const int per = (P + int(blockDim.x) - 1) / int(blockDim.x);
    const int lo = int(threadIdx.x) * per;
    const int hi = min(P, lo + per);
    int sum = 0;
    for (int i = lo; i < hi; ++i) sum += count[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int t = 0; t < int(blockDim.x); ++t) {
            const int v = part[t];
            part[t] = acc;
            acc += v;
        }
    }
    __syncthreads();
    int acc = part[threadIdx.x];
    for (int i = lo; i < hi; ++i) {
        start[i] = acc;
        cursor[i] = acc;
        acc += count[i];
    }
}

// perm[position] = row, rows grouped by bucket (the order inside a bucket is
// whatever the atomics give: the results do not depend on it)
__global__ void bucket_scatter_kernel(const uint32_t *__restrict__ pivot, int64_t n, int *__restrict__ cursor,
                                      uint32_t *__restrict__ perm) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int pos = atomicAdd(cursor + pivot[i], 1);
    perm[pos] = uint32_t(i);
}

// rot[x] = the database tile where query tile x's scan starts: the tile
// holding the first position of the bucket of the tile's first row
__global__ void scan_rotation_kernel(const uint32_t *__restrict__ perm, const uint32_t *__restrict__ pivot,
                                     const int *__restrict__ start, int64_t qtiles, int *__restrict__ rot) {
    const int64_t x = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (x >= qtiles) return;
    rot[x] = start[pivot[perm[x * TILE]]] / TILE;
}

constexpr size_t kMaxSmem = 227 * 1024;

}  // namespace

// ---------------------------------------------------------------------------
// Host entry points.
// ---------------------------------------------------------------------------
int tc_padded_k(int64_t dim) { return int((dim + KBE - 1) / KBE * KBE); }
int tc_segments_per_split(int qt) { return qt == 1 ? col_splits<1>() : col_splits<2>(); }
int64_t tc_tiles(int64_t rows) { return (rows + TILE - 1) / TILE; }
size_t tc_tile_bytes(int64_t dim) { return size_t(TILE) * tc_padded_k(dim) * 2; }

// Picks (query tiles per CTA, stages) for this K and candidate count.
// Ring depth (K-block stages) of the wide scan for this K and candidate
// count; false if fewer than three stages fit next to the heaps.
bool wide_choose(int kp, int kk, int *kst);
bool tc_wide_fits(int kp, int kk) {
    int kst = 0;
    return wide_choose(kp, kk, &kst);
}
int tc_wide_stages(int kp, int kk) {
    int kst = 0;
    return wide_choose(kp, kk, &kst) ? kst : 0;
}
bool pair_choose(int kp, int kk, int *kst);
bool tc_pair_fits(int kp, int kk) {
    int kst = 0;
    return pair_choose(kp, kk, &kst);
}
// Ring depth of the pair scan (8 KB stages); false if fewer than four fit.
bool pair_choose(int kp, int kk, int *kst) {
    if (PairSmem<12>::total(kp, kk) <= kMaxSmem) { *kst = 12; return true; }
    if (PairSmem<10>::total(kp, kk) <= kMaxSmem) { *kst = 10; return true; }
    if (PairSmem<8>::total(kp, kk) <= kMaxSmem) { *kst = 8; return true; }
    if (PairSmem<6>::total(kp, kk) <= kMaxSmem) { *kst = 6; return true; }
    if (PairSmem<4>::total(kp, kk) <= kMaxSmem) { *kst = 4; return true; }
    return false;
}
// Ring depth of the one-heap-per-query pair scan (long candidate lists).
bool pair1_choose(int kp, int kk, int *kst) {
    if (PairSmem<12, 1>::total(kp, kk) <= kMaxSmem) { *kst = 12; return true; }
    if (PairSmem<10, 1>::total(kp, kk) <= kMaxSmem) { *kst = 10; return true; }
    if (PairSmem<8, 1>::total(kp, kk) <= kMaxSmem) { *kst = 8; return true; }
    if (PairSmem<6, 1>::total(kp, kk) <= kMaxSmem) { *kst = 6; return true; }
    if (PairSmem<4, 1>::total(kp, kk) <= kMaxSmem) { *kst = 4; return true; }
    return false;
}
bool tc_long_fits(int kp, int kk) {
    int kst = 0;
    return pair1_choose(kp, kk, &kst);
}

bool wide_choose(int kp, int kk, int *kst) {
    if (WideSmem<5>::total(kp, kk) <= kMaxSmem) { *kst = 5; return true; }
    if (WideSmem<4>::total(kp, kk) <= kMaxSmem) { *kst = 4; return true; }
    if (WideSmem<3>::total(kp, kk) <= kMaxSmem) { *kst = 3; return true; }
    return false;
}

bool tc_choose(int kp, int kk, int *qt, int *stages) {
    // One query tile per CTA with eight epilogue warps measured faster than two
    // query tiles with four warps each (the epilogue, not the database
    // traffic, limits the scan), so only QT = 1 is used.
    if (TcSmem<1, 4>::total(kp, kk) <= kMaxSmem) { *qt = 1; *stages = 4; return true; }
    if (TcSmem<1, 3>::total(kp, kk) <= kMaxSmem) { *qt = 1; *stages = 3; return true; }
    if (TcSmem<1, 2>::total(kp, kk) <= kMaxSmem) { *qt = 1; *stages = 2; return true; }
    return false;
}

cudaError_t launch_bf16_tiles(const float *x, int64_t rows, int64_t dim, int64_t tiles, uint8_t *out,
                              cudaStream_t st, int *launches, const uint32_t *map, int split) {
    const int kp = tc_padded_k(dim);
    const int64_t total = tiles * TILE * ((split ? 3 : 1) * kp / 8);
    int64_t blocks = (total + 255) / 256;
    if (blocks > 148 * 64) blocks = 148 * 64;
    if (blocks < 1) blocks = 1;
    if (launches) *launches += 1;
    bf16_tile_kernel<<<unsigned(blocks), 256, 0, st>>>(x, rows, int(dim), kp, split, tiles, map, out);
    return cudaGetLastError();
}

cudaError_t launch_tc_norms(int metric, const float *x, int64_t rows, int64_t dim, int64_t padded, float *out,
                            cudaStream_t st, int *launches, const uint32_t *map) {
    const int mc = metric_class(metric);
    if (launches) *launches += 1;
    tc_norm_kernel<<<unsigned((padded + 255) / 256), 256, 0, st>>>(x, rows, int(dim), padded, mc, map, out);
    return cudaGetLastError();
}

cudaError_t launch_tc_filter(int metric, const uint8_t *q_tiles, const uint8_t *d_tiles, const float *d_norm,
                             int64_t n, int64_t m, int64_t dim, int splits, const float *thr, uint64_t *fout,
                             int *fcount, int fcap, int *err, cudaStream_t st, int *launches) {
    TcArgs a{};
    a.qt = q_tiles;
    a.dt = d_tiles;
    a.dnorm = d_norm;
    a.n = n;
    a.m = m;
    a.kp = tc_padded_k(dim);
    a.kk = 0;
    a.splits = splits;
    a.n_tiles = tc_tiles(n);
    a.split_tiles = (a.n_tiles + splits - 1) / splits;
    a.err = err;
    a.thr = thr;
    a.fout = fout;
    a.fcount = fcount;
    a.fcap = fcap;
    // four ring stages, fewer for wide K (at K = 256 two fit)
    const int mc = metric_class(metric);
    if (TcSmem<1, 4>::total(a.kp, 0) <= kMaxSmem) {
        if (launches) *launches += 1;
        return launch_tc_mc<1, 4, true>(a, mc, st);
    }
    if (TcSmem<1, 3>::total(a.kp, 0) <= kMaxSmem) {
        if (launches) *launches += 1;
        return launch_tc_mc<1, 3, true>(a, mc, st);
    }
    if (TcSmem<1, 2>::total(a.kp, 0) > kMaxSmem) return cudaErrorInvalidValue;
    if (launches) *launches += 1;
    return launch_tc_mc<1, 2, true>(a, mc, st);
}

cudaError_t launch_sample_bound(const uint64_t *cand, int64_t m, int segs, int kk, float *thr, cudaStream_t st,
                                int *launches) {
    if (m <= 0) return cudaSuccess;
    if (launches) *launches += 1;
    sample_bound_kernel<<<unsigned((m + 255) / 256), 256, 0, st>>>(cand, m, segs, kk, thr);
    return cudaGetLastError();
}

cudaError_t launch_filter_select(const uint64_t *fout, const int *fcount, int64_t m, int fcap, int kk,
                                 uint64_t *cand, int *flags, int *flag_count, cudaStream_t st, int *launches) {
    if (m <= 0) return cudaSuccess;
    const size_t smem = size_t(next_pow2(fcap)) * 8;
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(filter_select_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    if (launches) *launches += 1;
    filter_select_kernel<<<unsigned(m), 256, smem, st>>>(fout, fcount, fcap, kk, cand, flags, flag_count);
    return cudaGetLastError();
}

cudaError_t launch_tc_scan(int metric, const uint8_t *q_tiles, const uint8_t *d_tiles, const float *d_norm,
                           int64_t n, int64_t m, int64_t dim, int kk, int splits, uint64_t *cand, int *err,
                           cudaStream_t st, int *launches, int *qt_out, const uint32_t *perm, const int *rot,
                           bool wide, int64_t wave, bool pair, uint32_t *qbound) {
    // (qt_out receives the query tiles per CTA; segments per split follow from it)
    TcArgs a{};
    a.qt = q_tiles;
    a.dt = d_tiles;
    a.dnorm = d_norm;
    a.n = n;
    a.m = m;
    a.kp = tc_padded_k(dim);
    a.kk = kk;
    a.splits = splits;
    a.n_tiles = tc_tiles(n);
    a.split_tiles = (a.n_tiles + splits - 1) / splits;
    a.cand = cand;
    a.err = err;
    a.perm = perm;
    a.rot = rot;
    a.qbound = qbound;
    int qt = 1, stages = 0, kst = 0, pkst = 0;
    // CTA pairs when asked for, or when the one-CTA wide scan does not fit
    // (their ring stages are half the size)
    const bool wide_ok = wide && wide_choose(a.kp, kk, &kst);
    const bool use_pair = wide && (pair || !wide_ok) && pair_choose(a.kp, kk, &pkst);
    const bool use_wide = !use_pair && wide_ok;
    if (!use_pair && !use_wide && !tc_choose(a.kp, kk, &qt, &stages)) return cudaErrorInvalidValue;
    if ((perm || rot) && qt != 1) return cudaErrorInvalidValue;
    if (qt_out) *qt_out = qt;
    const int mc = metric_class(metric);
    if (use_pair) {
        if (pkst == 12) return launch_pair_mc<12>(a, mc, st, wave, launches);
        if (pkst == 10) return launch_pair_mc<10>(a, mc, st, wave, launches);
        if (pkst == 8) return launch_pair_mc<8>(a, mc, st, wave, launches);
        if (pkst == 6) return launch_pair_mc<6>(a, mc, st, wave, launches);
        return launch_pair_mc<4>(a, mc, st, wave, launches);
    }
    if (use_wide) {
        if (kst == 5) return launch_wide_mc<5>(a, mc, st, wave, launches);
        if (kst == 4) return launch_wide_mc<4>(a, mc, st, wave, launches);
        return launch_wide_mc<3>(a, mc, st, wave, launches);
    }
    if (launches) *launches += 1;
    if (stages == 4) return launch_tc_mc<1, 4>(a, mc, st);
    if (stages == 3) return launch_tc_mc<1, 3>(a, mc, st);
    return launch_tc_mc<1, 2>(a, mc, st);
}

cudaError_t launch_tc_scan_long(int metric, const uint8_t *q_tiles, const uint8_t *d_tiles, const float *d_norm,
                                int64_t n, int64_t m, int64_t dim, int kk, int splits, uint64_t *cand, int *err,
                                cudaStream_t st, int *launches, const uint32_t *perm, const int *rot, int64_t wave,
                                uint32_t *qbound) {
    TcArgs a{};
    a.qt = q_tiles;
    a.dt = d_tiles;
    a.dnorm = d_norm;
    a.n = n;
    a.m = m;
    a.kp = tc_padded_k(dim);
    a.kk = kk;
    a.splits = splits;
    a.n_tiles = tc_tiles(n);
    a.split_tiles = (a.n_tiles + splits - 1) / splits;
    a.cand = cand;
    a.err = err;
    a.perm = perm;
    a.rot = rot;
    a.qbound = qbound;
    int kst = 0;
    if (!pair1_choose(a.kp, kk, &kst)) return cudaErrorInvalidValue;
    const int mc = metric_class(metric);
    if (kst == 12) return launch_pair_mc<12, 1>(a, mc, st, wave, launches);
    if (kst == 10) return launch_pair_mc<10, 1>(a, mc, st, wave, launches);
    if (kst == 8) return launch_pair_mc<8, 1>(a, mc, st, wave, launches);
    if (kst == 6) return launch_pair_mc<6, 1>(a, mc, st, wave, launches);
    return launch_pair_mc<4, 1>(a, mc, st, wave, launches);
}

cudaError_t launch_locality_order(const uint64_t *cand, int64_t n, int segs, int P, const uint32_t *rank,
                                  uint32_t *pivot, int *count, int *start, int *cursor, uint32_t *perm, int *rot,
                                  cudaStream_t st, int *launches) {
    if (P < 1 || P > 1024 * 64) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(count, 0, size_t(P) * sizeof(int), st);
    if (e != cudaSuccess) return e;
    const unsigned nb = unsigned((n + 255) / 256);
    nearest_pivot_kernel<<<nb, 256, 0, st>>>(cand, n, segs, rank, pivot, count);
    bucket_offsets_kernel<<<1, 1024, 0, st>>>(count, P, start, cursor);
    bucket_scatter_kernel<<<nb, 256, 0, st>>>(pivot, n, cursor, perm);
    const int64_t qtiles = tc_tiles(n);
    scan_rotation_kernel<<<unsigned((qtiles + 255) / 256), 256, 0, st>>>(perm, pivot, start, qtiles, rot);
    if (launches) *launches += 4;
    return cudaGetLastError();
}

}  // namespace ssg
