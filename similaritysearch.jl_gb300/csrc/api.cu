// api.cu -- the C ABI of libssgpu (declared in include/ssgpu.h).
//
// An index owns a device copy of the database, its CUDA stream, scratch
// buffers and a last-error string.  Every entry point validates its arguments
// the way the reference does (searchbatch! throws ArgumentError on an empty
// query set or mismatched output shape, src/SimilaritySearch.jl:334-335;
// allknn! asserts 0 < k <= n, src/allknn.jl:73-75) and returns a status code
// instead of throwing.  Nothing here falls back to a CPU path: every result is
// produced by the kernels in this library.
#include "ssgpu.h"
#include "common.cuh"
#include "kernels.h"
#include "chain.h"

#include <cuda_runtime.h>
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <vector>

namespace {

thread_local char g_err[512] = "";

// A device allocation owned by one object: freed by release() or when the
// object goes out of scope (temporaries of a call free their memory on every
// return path), never copied.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    cudaError_t ensure(size_t want) {
        if (want <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
};

bool is_sq_metric(int metric) { return metric == SSG_METRIC_SQL2 || metric == SSG_METRIC_L2; }

size_t elem_size(int e) {
    switch (e) {
        case SSG_ELEM_F32: return 4;
        case SSG_ELEM_U64: return 8;
        case SSG_ELEM_F64: return 8;
        case SSG_ELEM_F16: return 2;
        case SSG_ELEM_U8: return 1;
        case SSG_ELEM_I8: return 1;
        default: return 0;
    }
}

}  // namespace

struct ssg_index {
    int metric = 0, elem = 0, prec = 0;
    int64_t dim = 0, n = 0, cap = 0;
    int device = 0;
    DevBuf db;       // n x dim Float32 rows, or n x W UInt64 sketches
    DevBuf db_norm;  // |x| per row (COSINE)
    DevBuf qbuf, qnorm, qraw, cand, gheap, outbuf, stage;
    // BF16 tensor-core mode: operand tiles of the database and the queries,
    // per-row norms of the padded database, and the device status word.
    DevBuf tc_db, tc_norm, tc_q, status;
    // allknn's locality order (tc_bf16.cu): position -> id, start tile of
    // each query tile's scan, BF16 tiles and norms in that order; built for
    // loc_n rows (-1: none) from a pivot per loc_rows_param rows, the groups
    // in the pivots' chain order (loc_chain_param) or in pivot order
    DevBuf loc_perm, loc_rot, loc_tiles, loc_norm;
    int64_t loc_n = -1, loc_bf16_n = -1;
    int64_t loc_rows_param = 128;
    int loc_chain_param = 1;
    // the plain method's split tiles (both roles) and |x|^2 in that order,
    // built for loc_ps_n rows (-1: none)
    DevBuf loc_ps_db, loc_ps_dbq, loc_ps_norm;
    int64_t loc_ps_n = -1;
    int locality_param = 1;
    int wide_param = 1;    // BF16 scan: 256-row database tiles per MMA
    int64_t wave_param = 0;  // wide scan: query tiles per launch (0: one launch)
    int pair_param = 0;      // wide scan on CTA pairs (M = 256 MMAs, half the database traffic per SM)
    int long_param = 1;      // lists too long for two heaps per query: one heap per query on CTA pairs
    // K-streaming tensor-core path (FP8 mode, and BF16 for dim > 256): operand
    // tiles, per-row FP8 scales, per-row epilogue coefficients, query tiles
    DevBuf st_db, st_scale, st_alpha, st_beta, st_q, st_qscale;
    // plain FP32 GEMM-form path: |x|^2 per row and its maximum, query flags of
    // the completeness check and the fallback's buffers
    DevBuf sq_norm, sq_max, flags, qsq, fb_list, fb_q, fb_out, fb_cand, fb_qn;
    // BF16 threshold-filter path (candidate counts beyond the on-chip heaps):
    // tiles of every smp_r-th database row, filtered lists, counts, bounds
    DevBuf tc_smp, tc_smp_norm, f_out, f_cnt, f_thr, gbound;
    DevBuf pack_q, pack_out;  // ssg_search_batches staging
    DevBuf qbound;            // per-query bounds shared by a query's split heaps (ScanArgs::qbound)
    // plain GEMM-form scan: k-major tiles of the database (built for gm_rows
    // rows) and of the current queries
    DevBuf gm_db, gm_q;
    int64_t gm_rows = -1;
    // the plain method on the tensor cores: two-piece BF16 tiles of the
    // database in the database role (ps_db, with |x|^2 per padded row in
    // ps_norm) and, for allknn, in the query role (ps_dbq), built for
    // ps_rows rows; the current queries' tiles (ps_q)
    DevBuf ps_db, ps_dbq, ps_norm, ps_q;
    int64_t ps_rows = -1, ps_qrows = -1;
    // the same for wide vectors in the K-streaming layout: split tiles of the
    // database (both roles), its epilogue coefficients, the queries' tiles
    DevBuf pss_db, pss_dbq, pss_alpha, pss_beta, pss_q;
    int64_t pss_rows = -1, pss_qrows = -1;
    int plain_tc_param = 1;
    int last_plain_tc = 0;  // 1: the last plain-method search ran on the tensor cores
    int64_t smp_r = 0, smp_n = -1, smp_rows = 0;
    DevBuf red[2];  // segment-reduction passes (merge_groups) ping-pong
    // learned shortlist (trained model, whether searches use it, recall target)
    ssg::LearnedModel *learned = nullptr;
    int learned_param = 1;
    double learned_target = 0.99;
    double train_hard = 0.5;  // share of semi-hard negatives in training triplets
    int last_learned = 0;
    float max_x_sq = 0.0f;
    int margin_param = 0;
    int exact_scan_param = 0;
    int plain_param = 0;  // 1: run the plain FP32 method on a reduced-precision index
    int last_fallbacks = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::mutex mu;
    char err[512] = "";
    // tunables
    int splits_param = 0;
    double overfetch = 4.0;
    int profile = 0;
    // statistics
    double main_ms = 0.0;
    int64_t main_launches = 0;
    int last_launches = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // CUDA graphs of ssg_search_batches' device work, one per shape: the
    // first call of a shape runs eagerly (sizing every buffer), the second is
    // captured on cap_stream and every later one replays the graph
    struct GraphEntry {
        cudaGraphExec_t exec;
        int launches;
    };
    int graphs_param = 1;
    bool capturing = false;
    cudaStream_t cap_stream = nullptr;
    std::map<std::vector<uint64_t>, GraphEntry> graphs;
    std::set<std::vector<uint64_t>> graph_seen;
    int64_t graph_replays = 0;
    int last_graph = 0;
};

namespace {

int fail(ssg_index *idx, int code, const char *fmt, ...) {
    char *dst = idx ? idx->err : g_err;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(dst, 512, fmt, ap);
    va_end(ap);
    return code;
}

int cuda_fail(ssg_index *idx, cudaError_t e, const char *what) {
    cudaGetLastError();  // clear the sticky-free error state of the last call
    return fail(idx, e == cudaErrorMemoryAllocation ? SSG_ENOMEM : SSG_ECUDA, "%s: %s (%s)", what,
                cudaGetErrorString(e), cudaGetErrorName(e));
}

#define SSG_CK(call, what)                                  \
    do {                                                    \
        cudaError_t _e = (call);                            \
        if (_e != cudaSuccess) return cuda_fail(idx, _e, what); \
    } while (0)

// Uploads `rows` rows (row stride `ld` elements of `elem`) from host or device
// memory into dst as contiguous Float32 (or UInt64) rows of `dim`.
int upload_rows(ssg_index *idx, void *dst, const void *src, int64_t rows, int64_t ld, bool src_device) {
    if (rows == 0) return SSG_OK;
    const size_t es = elem_size(idx->elem);
    const cudaMemcpyKind kind = src_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const bool cast = (idx->elem != SSG_ELEM_F32 && idx->elem != SSG_ELEM_U64);
    void *target = dst;
    if (cast) {
        SSG_CK(idx->stage.ensure(size_t(rows) * idx->dim * es), "allocating the cast staging buffer");
        target = idx->stage.p;
    }
    if (ld == idx->dim) {
        SSG_CK(cudaMemcpyAsync(target, src, size_t(rows) * idx->dim * es, kind, idx->stream), "copying rows");
    } else {
        SSG_CK(cudaMemcpy2DAsync(target, size_t(idx->dim) * es, src, size_t(ld) * es,
                                 size_t(idx->dim) * es, size_t(rows), kind, idx->stream),
               "copying strided rows");
    }
    if (cast) {
        SSG_CK(ssg::launch_cast_f32(idx->stage.p, idx->elem, rows * idx->dim, static_cast<float *>(dst),
                                    idx->stream, &idx->last_launches),
               "casting rows to Float32");
    }
    return SSG_OK;
}

int ensure_db_capacity(ssg_index *idx, int64_t rows) {
    if (rows <= idx->cap) return SSG_OK;
    int64_t newcap = std::max<int64_t>(rows, idx->cap + idx->cap / 2);
    const size_t row_bytes = size_t(idx->dim) * (idx->metric == SSG_METRIC_HAMMING ? 8 : 4);
    void *p = nullptr;
    SSG_CK(cudaMalloc(&p, size_t(newcap) * row_bytes), "allocating the database");
    if (idx->n > 0) {
        cudaError_t e = cudaMemcpyAsync(p, idx->db.p, size_t(idx->n) * row_bytes, cudaMemcpyDeviceToDevice,
                                        idx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(idx->stream);
        if (e != cudaSuccess) {
            cudaFree(p);
            return cuda_fail(idx, e, "growing the database");
        }
    }
    idx->db.release();
    idx->db.p = p;
    idx->db.bytes = size_t(newcap) * row_bytes;
    if (idx->metric == SSG_METRIC_COSINE) {
        void *np = nullptr;
        SSG_CK(cudaMalloc(&np, size_t(newcap) * 4), "allocating database norms");
        if (idx->n > 0) {
            cudaError_t e = cudaMemcpyAsync(np, idx->db_norm.p, size_t(idx->n) * 4, cudaMemcpyDeviceToDevice,
                                            idx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(idx->stream);
            if (e != cudaSuccess) {
                cudaFree(np);
                return cuda_fail(idx, e, "growing database norms");
            }
        }
        idx->db_norm.release();
        idx->db_norm.p = np;
        idx->db_norm.bytes = size_t(newcap) * 4;
    }
    idx->cap = newcap;
    return SSG_OK;
}

// (Re)builds the BF16 operand tiles and row norms of the whole database.
// Tiles are allocated in pairs so a CTA holding two query tiles never reads
// past the end when the database doubles as the query set (allknn).
int build_tc_tiles(ssg_index *idx) {
    idx->loc_n = -1;
    idx->loc_bf16_n = -1;
    idx->loc_ps_n = -1;
    const int64_t tiles = (ssg::tc_tiles(idx->n) + 1) / 2 * 2;
    const size_t tb = ssg::tc_tile_bytes(idx->dim);
    SSG_CK(idx->tc_db.ensure(size_t(tiles) * tb), "allocating BF16 database tiles");
    SSG_CK(ssg::launch_bf16_tiles(static_cast<const float *>(idx->db.p), idx->n, idx->dim, tiles,
                                  static_cast<uint8_t *>(idx->tc_db.p), idx->stream, &idx->last_launches),
           "building BF16 database tiles");
    SSG_CK(idx->tc_norm.ensure(size_t(tiles) * 128 * 4), "allocating BF16 row norms");
    SSG_CK(ssg::launch_tc_norms(idx->metric, static_cast<const float *>(idx->db.p), idx->n, idx->dim, tiles * 128,
                                static_cast<float *>(idx->tc_norm.p), idx->stream, &idx->last_launches),
           "computing BF16 row norms");
    SSG_CK(cudaStreamSynchronize(idx->stream), "building BF16 tiles");
    return SSG_OK;
}

// The resident-query BF16 kernel holds a query tile on chip (dim <= 256);
// FP8 and wider BF16 stream both operands along K.
bool uses_stream(const ssg_index *idx) {
    return idx->prec == SSG_PREC_FP8 || (idx->prec == SSG_PREC_BF16 && ssg::tc_padded_k(idx->dim) > 256);
}

// (Re)builds the K-block operand tiles, FP8 scales and epilogue coefficients.
int build_stream_tiles(ssg_index *idx) {
    const int fp8 = idx->prec == SSG_PREC_FP8;
    const int64_t tiles = ssg::tc_tiles(idx->n);
    SSG_CK(idx->st_db.ensure(size_t(tiles) * ssg::stream_tile_bytes(idx->dim, fp8)), "allocating operand tiles");
    float *scale = nullptr;
    if (fp8) {
        SSG_CK(idx->st_scale.ensure(size_t(tiles) * 128 * 4), "allocating FP8 scales");
        scale = static_cast<float *>(idx->st_scale.p);
    }
    SSG_CK(ssg::launch_stream_tiles(static_cast<const float *>(idx->db.p), idx->n, idx->dim, fp8, tiles,
                                    static_cast<uint8_t *>(idx->st_db.p), scale, idx->stream, &idx->last_launches),
           "building operand tiles");
    SSG_CK(idx->st_alpha.ensure(size_t(tiles) * 128 * 4), "allocating epilogue coefficients");
    SSG_CK(idx->st_beta.ensure(size_t(tiles) * 128 * 4), "allocating epilogue coefficients");
    SSG_CK(ssg::launch_stream_coefs(idx->metric, static_cast<const float *>(idx->db.p), idx->n, idx->dim, tiles * 128,
                                    scale, static_cast<float *>(idx->st_alpha.p), static_cast<float *>(idx->st_beta.p),
                                    idx->stream, &idx->last_launches),
           "computing epilogue coefficients");
    SSG_CK(cudaStreamSynchronize(idx->stream), "building operand tiles");
    return SSG_OK;
}

int add_rows(ssg_index *idx, const void *src, int64_t rows, int64_t ld, bool src_device) {
    int rc = ensure_db_capacity(idx, idx->n + rows);
    if (rc) return rc;
    const size_t row_bytes = size_t(idx->dim) * (idx->metric == SSG_METRIC_HAMMING ? 8 : 4);
    void *dst = static_cast<char *>(idx->db.p) + size_t(idx->n) * row_bytes;
    rc = upload_rows(idx, dst, src, rows, ld, src_device);
    if (rc) return rc;
    if (idx->metric == SSG_METRIC_COSINE) {
        SSG_CK(ssg::launch_row_norms(static_cast<const float *>(dst), rows, idx->dim,
                                     static_cast<float *>(idx->db_norm.p) + idx->n, idx->stream,
                                     &idx->last_launches),
               "computing database norms");
    }
    SSG_CK(cudaStreamSynchronize(idx->stream), "uploading the database");
    idx->n += rows;
    if (is_sq_metric(idx->metric) && idx->n > 0) {
        // |x|^2 per row (GEMM-form SqL2) and its maximum (completeness bound)
        SSG_CK(idx->sq_norm.ensure(size_t(idx->n) * 4), "allocating squared norms");
        SSG_CK(idx->sq_max.ensure(16), "allocating the norm maximum");
        SSG_CK(cudaMemsetAsync(idx->sq_max.p, 0, 4, idx->stream), "clearing the norm maximum");
        SSG_CK(ssg::launch_row_sq_norms(static_cast<const float *>(idx->db.p), idx->n, idx->dim,
                                        static_cast<float *>(idx->sq_norm.p), static_cast<float *>(idx->sq_max.p),
                                        idx->stream, &idx->last_launches),
               "computing squared norms");
        SSG_CK(cudaMemcpyAsync(&idx->max_x_sq, idx->sq_max.p, 4, cudaMemcpyDeviceToHost, idx->stream),
               "reading the norm maximum");
        SSG_CK(cudaStreamSynchronize(idx->stream), "computing squared norms");
    }
    if (idx->prec != SSG_PREC_FP32) {
        rc = uses_stream(idx) ? build_stream_tiles(idx) : build_tc_tiles(idx);
        if (rc) return rc;
    }
    return SSG_OK;
}

int validate_create(int metric, int elem, int64_t dim, int64_t n, int64_t ld, int prec) {
    if (metric < SSG_METRIC_SQL2 || metric > SSG_METRIC_HAMMING)
        return fail(nullptr, SSG_EUNSUPPORTED, "unsupported metric code %d", metric);
    if (elem_size(elem) == 0) return fail(nullptr, SSG_EUNSUPPORTED, "unsupported element type %d", elem);
    if (metric == SSG_METRIC_HAMMING && elem != SSG_ELEM_U64)
        return fail(nullptr, SSG_EUNSUPPORTED, "Hamming needs UInt64 sketches (element type %d given)", elem);
    if (metric != SSG_METRIC_HAMMING && elem == SSG_ELEM_U64)
        return fail(nullptr, SSG_EUNSUPPORTED, "float metrics need a numeric element type, not UInt64");
    if (dim <= 0) return fail(nullptr, SSG_EINVAL, "dimension must be positive (got %lld)", (long long)dim);
    if (metric == SSG_METRIC_HAMMING && dim > 32)
        return fail(nullptr, SSG_EUNSUPPORTED, "Hamming sketches are limited to 32 words (2048 bits), got %lld",
                    (long long)dim);
    if (n < 0 || n >= (int64_t(1) << 32) - 1)
        return fail(nullptr, SSG_EINVAL, "database length %lld out of range", (long long)n);
    if (ld < dim) return fail(nullptr, SSG_EINVAL, "leading dimension %lld < dim %lld", (long long)ld, (long long)dim);
    if (prec != SSG_PREC_FP32 && prec != SSG_PREC_BF16 && prec != SSG_PREC_FP8)
        return fail(nullptr, SSG_EUNSUPPORTED, "precision mode %d is not supported", prec);
    if (prec != SSG_PREC_FP32 && metric == SSG_METRIC_HAMMING)
        return fail(nullptr, SSG_EUNSUPPORTED, "Hamming distances are integers: only the exact mode exists");
    return SSG_OK;
}

int create_common(int metric, int elem, int64_t dim, int64_t n, const void *src, int64_t ld, int prec,
                  ssg_index **out, bool src_device) {
    if (!out) return fail(nullptr, SSG_EINVAL, "out pointer is NULL");
    *out = nullptr;
    int rc = validate_create(metric, elem, dim, n, ld, prec);
    if (rc) return rc;
    if (n > 0 && !src) return fail(nullptr, SSG_EINVAL, "database pointer is NULL");
    ssg_index *idx = new ssg_index();
    idx->metric = metric;
    idx->elem = elem;
    idx->prec = prec;
    idx->dim = dim;
    cudaError_t e = cudaGetDevice(&idx->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&idx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&idx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&idx->ev1);
    if (e != cudaSuccess) {
        cuda_fail(nullptr, e, "creating the index stream");
        ssg_destroy(idx);
        return SSG_ECUDA;
    }
    idx->own_stream = true;
    rc = add_rows(idx, src, n, ld, src_device);
    if (rc) {
        snprintf(g_err, sizeof g_err, "%s", idx->err);
        ssg_destroy(idx);
        return rc;
    }
    *out = idx;
    return SSG_OK;
}

// Picks the number of database splits per query tile: enough blocks to fill
// the GPU several times over, while every split stays long enough to amortise
// its heap and the merge stays within one block's shared memory.
// Database splits per query tile for a kernel with `cap` resident CTAs on the
// device: qctas * s CTAs run in ceil(qctas * s / cap) waves, each CTA scanning
// 1/s of the database, so the scan takes ~ waves(s) / s.  Minimise that, with
// a 1% charge per extra split for the wider merge, over s <= max_s.
int64_t wave_splits(int64_t qctas, int64_t cap, int64_t max_s) {
    qctas = std::max<int64_t>(1, qctas);
    const int64_t hi = std::max<int64_t>(1, std::min<int64_t>(max_s, 4 * ((cap + qctas - 1) / qctas)));
    int64_t best = 1;
    double best_cost = 1e300;
    for (int64_t sp = 1; sp <= hi; ++sp) {
        const double waves = double((qctas * sp + cap - 1) / cap);
        const double cost = waves / double(sp) * (1.0 + 0.01 * double(sp - 1));
        if (cost < best_cost * (1.0 - 1e-9)) { best_cost = cost; best = sp; }
    }
    return best;
}

int choose_splits(ssg_index *idx, int64_t m, int kk, int qpb) {
    if (idx->splits_param > 0) return idx->splits_param;
    const int64_t qtiles = (m + qpb - 1) / qpb;
    const int64_t target = int64_t(4) * ssg::device_sm_count();
    int64_t s = (target + qtiles - 1) / qtiles;
    const int64_t min_len = std::max<int64_t>(1024, int64_t(8) * kk);
    s = std::min<int64_t>(s, std::max<int64_t>(1, idx->n / min_len));
    return int(std::max<int64_t>(1, s));
}

// Records the scan kernel's duration when profiling (events around it on the
// index's stream).
struct ScanTimer {
    ssg_index *idx;
    explicit ScanTimer(ssg_index *i) : idx(i) {}
    int begin() {
        if (idx->profile) SSG_CK(cudaEventRecord(idx->ev0, idx->stream), "recording an event");
        return SSG_OK;
    }
    int end() {
        if (idx->profile) SSG_CK(cudaEventRecord(idx->ev1, idx->stream), "recording an event");
        return SSG_OK;
    }
    int collect() {
        if (!idx->profile) return SSG_OK;
        SSG_CK(cudaEventSynchronize(idx->ev1), "timing the scan kernel");
        float ms = 0.f;
        SSG_CK(cudaEventElapsedTime(&ms, idx->ev0, idx->ev1), "timing the scan kernel");
        idx->main_ms += ms;
        idx->main_launches += 1;
        return SSG_OK;
    }
};

#define SSG_RC(call)        \
    do {                    \
        int _rc = (call);   \
        if (_rc) return _rc; \
    } while (0)

// Reduces each query's `segs` sorted candidate segments (kk keys each) by
// merge passes until one merge block holds them; returns the buffer and the
// segment count the final merge should read.
int reduce_segments(ssg_index *idx, const uint64_t *cand, int64_t m, int segs, int kk, const uint64_t **out,
                    int *out_segs) {
    const uint64_t *cur = cand;
    int cs = segs;
    int which = 0;
    while (int64_t(cs) * kk > ssg::kMergeKeys) {
        const int group = std::max(2, ssg::kMergeKeys / kk);
        const int ns = (cs + group - 1) / group;
        DevBuf &b = idx->red[which];
        SSG_CK(b.ensure(size_t(m) * ns * kk * 8), "allocating merge scratch");
        SSG_CK(ssg::launch_merge_groups(cur, m, cs, kk, group, static_cast<uint64_t *>(b.p), idx->stream,
                                        &idx->last_launches),
               "launching a merge pass");
        cur = static_cast<const uint64_t *>(b.p);
        cs = ns;
        which ^= 1;
    }
    *out = cur;
    *out_segs = cs;
    return SSG_OK;
}

// The exact scan (direct FP32 or Hamming) then merge and decode.  dq are
// device query rows (Float32 or UInt64), dqn their norms (Cosine).  self_ids
// (device, optional) names each query's own object for exclude_self when the
// queries are not the contiguous range 0..m-1 of the database.
int run_exact_scan(ssg_index *idx, const void *dq, const float *dqn, int64_t m, int k, int exclude_self,
                   const int64_t *self_ids, uint32_t *d_ids, float *d_dists, DevBuf &cand) {
    const int take = k + (exclude_self ? 1 : 0);
    const int kk = int(std::min<int64_t>(take, std::max<int64_t>(1, idx->n)));
    const int splits = choose_splits(idx, m, kk, 128);
    const int64_t split_len = (idx->n + splits - 1) / splits;
    // bound the candidate scratch to ~1 GiB by processing queries in chunks
    const size_t per_query = size_t(splits) * kk * 8;
    int64_t chunk = std::max<int64_t>(1, int64_t((size_t(1) << 30) / per_query));
    chunk = std::min<int64_t>(chunk, m);
    SSG_CK(cand.ensure(per_query * size_t(chunk)), "allocating candidate scratch");
    const size_t qrow_bytes = size_t(idx->dim) * (idx->metric == SSG_METRIC_HAMMING ? 8 : 4);
    ScanTimer timer(idx);
    for (int64_t c0 = 0; c0 < m; c0 += chunk) {
        const int64_t mc = std::min<int64_t>(chunk, m - c0);
        ssg::ScanArgs a{};
        a.metric = idx->metric;
        a.n = idx->n;
        a.dim = idx->dim;
        a.m = mc;
        a.kk = kk;
        a.splits = splits;
        a.split_len = split_len;
        a.cand = static_cast<uint64_t *>(cand.p);
        a.id_base = 0;
        const void *qc = static_cast<const char *>(dq) + size_t(c0) * qrow_bytes;
        if (splits > 1) {
            // the splits of a query share one bound (all ones: none yet)
            SSG_CK(idx->qbound.ensure(size_t(chunk) * 4), "allocating query bounds");
            SSG_CK(cudaMemsetAsync(idx->qbound.p, 0xff, size_t(mc) * 4, idx->stream), "clearing query bounds");
            a.qbound = static_cast<uint32_t *>(idx->qbound.p);
        }
        size_t gh = idx->metric == SSG_METRIC_HAMMING ? ssg::hamming_gheap_bytes(a) : ssg::direct_gheap_bytes(a);
        if (gh) {
            SSG_CK(idx->gheap.ensure(gh), "allocating heap scratch");
            a.gheap = static_cast<uint64_t *>(idx->gheap.p);
        }
        SSG_RC(timer.begin());
        cudaError_t e;
        if (idx->metric == SSG_METRIC_HAMMING) {
            e = ssg::launch_hamming(a, static_cast<const uint64_t *>(idx->db.p), static_cast<const uint64_t *>(qc),
                                    idx->stream, &idx->last_launches);
        } else {
            e = ssg::launch_direct_f32(a, static_cast<const float *>(idx->db.p),
                                       static_cast<const float *>(idx->db_norm.p), static_cast<const float *>(qc),
                                       dqn ? dqn + c0 : nullptr, idx->stream, &idx->last_launches);
        }
        SSG_CK(e, "launching the scan kernel");
        SSG_RC(timer.end());
        ssg::FinalizeArgs f{};
        SSG_RC(reduce_segments(idx, a.cand, mc, splits, kk, &f.cand, &f.segs));
        f.kk = kk;
        f.m = mc;
        f.k_out = k;
        f.exclude_self = exclude_self;
        f.self_base = c0;
        f.self_ids = self_ids ? self_ids + c0 : nullptr;
        f.out_ids = d_ids + size_t(c0) * k;
        f.out_dists = d_dists + size_t(c0) * k;
        SSG_CK(ssg::launch_finalize(f, idx->stream, &idx->last_launches), "launching the merge kernel");
        SSG_RC(timer.collect());
    }
    return SSG_OK;
}

// Candidates kept by the GEMM-form scan for SqL2 / L2 beyond the k needed.
int gemm_margin(const ssg_index *idx, int take) {
    return idx->margin_param > 0 ? idx->margin_param : std::max(8, (take + 3) / 4);
}

// The plain FP32 method through the register-tiled GEMM-form scan.  Dot
// metrics get exact keys directly; SqL2 / L2 re-score kk = k + margin
// candidates exactly, and queries whose margin is not provably enough are
// recomputed with the exact direct scan.
int run_fallback(ssg_index *idx, const float *dq, int64_t m, int k, int exclude_self, const int *flags, int nflag,
                 uint32_t *d_ids, float *d_dists);

int run_gemm(ssg_index *idx, const float *dq, const float *dqn, int64_t m, int k, int exclude_self,
             uint32_t *d_ids, float *d_dists, int kk) {
    const bool sq = is_sq_metric(idx->metric);
    const int64_t qtiles = (m + 127) / 128;
    int64_t splits = idx->splits_param > 0
                         ? idx->splits_param
                         : wave_splits(qtiles, int64_t(ssg::gemm_ctas_per_sm(kk)) * ssg::device_sm_count(),
                                       std::max<int64_t>(1, idx->n / 512));
    splits = std::min<int64_t>(splits, std::max<int64_t>(1, idx->n / 512));
    splits = std::max<int64_t>(1, splits);
    // splits of whole 128-row tiles
    const int64_t n_tiles = (idx->n + 127) / 128;
    const int64_t split_len = (n_tiles + splits - 1) / splits * 128;
    splits = (idx->n + split_len - 1) / split_len;
    const int segs = int(splits);
    const size_t per_query = size_t(segs) * kk * 8;
    int64_t chunk = std::max<int64_t>(128, int64_t((size_t(1) << 30) / per_query) / 128 * 128);
    chunk = std::min<int64_t>(chunk, m);
    SSG_CK(idx->cand.ensure(per_query * size_t(chunk)), "allocating candidate scratch");
    // k-major operand tiles: the database's (kept until it changes), the queries'
    const size_t tile_bytes = ssg::gemm_tile_floats(idx->dim) * 4;
    if (idx->gm_rows != idx->n) {
        SSG_CK(idx->gm_db.ensure(size_t(n_tiles) * tile_bytes), "allocating database tiles");
        SSG_CK(ssg::launch_gemm_tiles(static_cast<const float *>(idx->db.p), idx->n, idx->dim, n_tiles,
                                      static_cast<float *>(idx->gm_db.p), idx->stream, &idx->last_launches),
               "building database tiles");
        idx->gm_rows = idx->n;
    }
    const float *qtile_base = static_cast<const float *>(idx->gm_db.p);
    if (dq != idx->db.p) {
        SSG_CK(idx->gm_q.ensure(size_t(qtiles) * tile_bytes), "allocating query tiles");
        SSG_CK(ssg::launch_gemm_tiles(dq, m, idx->dim, qtiles, static_cast<float *>(idx->gm_q.p), idx->stream,
                                      &idx->last_launches),
               "building query tiles");
        qtile_base = static_cast<const float *>(idx->gm_q.p);
    }
    if (sq) {
        SSG_CK(idx->flags.ensure(size_t(m) * 4 + 16), "allocating query flags");
        SSG_CK(idx->qsq.ensure(size_t(chunk) * 4 + 16), "allocating query norms");
        SSG_CK(cudaMemsetAsync(idx->flags.p, 0, size_t(m) * 4 + 16, idx->stream), "clearing query flags");
    }
    int *flags = static_cast<int *>(idx->flags.p);
    int *flag_count = flags ? flags + m : nullptr;
    ScanTimer timer(idx);
    for (int64_t c0 = 0; c0 < m; c0 += chunk) {
        const int64_t mc = std::min<int64_t>(chunk, m - c0);
        ssg::ScanArgs a{};
        a.metric = idx->metric;
        a.n = idx->n;
        a.dim = idx->dim;
        a.m = mc;
        a.kk = kk;
        a.splits = int(splits);
        a.split_len = split_len;
        a.cand = static_cast<uint64_t *>(idx->cand.p);
        const float *qc = dq + size_t(c0) * idx->dim;
        const float *xaux = sq ? static_cast<const float *>(idx->sq_norm.p) : static_cast<const float *>(idx->db_norm.p);
        if (splits > 1) {
            // the splits of a query share one bound (all ones: none yet)
            SSG_CK(idx->qbound.ensure(size_t(chunk) * 4), "allocating query bounds");
            SSG_CK(cudaMemsetAsync(idx->qbound.p, 0xff, size_t(mc) * 4, idx->stream), "clearing query bounds");
            a.qbound = static_cast<uint32_t *>(idx->qbound.p);
        }
        SSG_RC(timer.begin());
        SSG_CK(ssg::launch_gemm_f32(a, static_cast<const float *>(idx->gm_db.p), xaux,
                                    qtile_base + size_t(c0 / 128) * ssg::gemm_tile_floats(idx->dim),
                                    dqn ? dqn + c0 : nullptr, idx->stream, &idx->last_launches),
               "launching the FP32 scan kernel");
        SSG_RC(timer.end());
        ssg::FinalizeArgs f{};
        SSG_RC(reduce_segments(idx, a.cand, mc, segs, kk, &f.cand, &f.segs));
        f.kk = kk;
        f.m = mc;
        f.k_out = k;
        f.exclude_self = exclude_self;
        f.self_base = c0;
        f.out_ids = d_ids + size_t(c0) * k;
        f.out_dists = d_dists + size_t(c0) * k;
        if (sq) {
            float *qsq = static_cast<float *>(idx->qsq.p);
            SSG_CK(ssg::launch_row_sq_norms(qc, mc, idx->dim, qsq, qsq + chunk, idx->stream, &idx->last_launches),
                   "computing query norms");
            f.check = 1;
            f.q_sq = qsq;
            f.max_x_sq = idx->max_x_sq;
            f.err_scale = 4.0f * float(idx->dim + 2) * 5.9604645e-8f;
            f.n_total = idx->n;
            f.flags = flags + c0;
            f.flag_count = flag_count;
            f.n_rows = idx->n;
            SSG_CK(ssg::launch_finalize_rerank(idx->metric, f, static_cast<const float *>(idx->db.p),
                                               static_cast<const float *>(idx->db_norm.p), idx->dim, qc,
                                               nullptr, idx->stream, &idx->last_launches),
                   "launching the rerank kernel");
        } else {
            SSG_CK(ssg::launch_finalize(f, idx->stream, &idx->last_launches), "launching the merge kernel");
        }
        SSG_RC(timer.collect());
    }
    if (!sq) return SSG_OK;
    // queries whose candidate margin was not provably sufficient
    int nflag = 0;
    SSG_CK(cudaMemcpyAsync(&nflag, flag_count, sizeof(int), cudaMemcpyDeviceToHost, idx->stream), "reading flags");
    SSG_CK(cudaStreamSynchronize(idx->stream), "running the FP32 scan");
    idx->last_fallbacks = nflag;
    return run_fallback(idx, dq, m, k, exclude_self, flags, nflag, d_ids, d_dists);
}

// Recomputes the flagged queries (flags[j] != 0, nflag of them) with the exact
// direct scan and scatters their rows into the results.
int run_fallback(ssg_index *idx, const float *dq, int64_t m, int k, int exclude_self, const int *flags, int nflag,
                 uint32_t *d_ids, float *d_dists) {
    if (nflag == 0) return SSG_OK;
    std::vector<int> hflags(static_cast<size_t>(m), 0);
    SSG_CK(cudaMemcpy(hflags.data(), flags, size_t(m) * 4, cudaMemcpyDeviceToHost), "reading flags");
    std::vector<int64_t> list;
    list.reserve(size_t(nflag));
    for (int64_t j = 0; j < m; ++j)
        if (hflags[size_t(j)]) list.push_back(j);
    const int64_t cnt = int64_t(list.size());
    const size_t row_bytes = size_t(idx->dim) * 4;
    SSG_CK(idx->fb_list.ensure(size_t(cnt) * 8), "allocating fallback list");
    SSG_CK(idx->fb_q.ensure(size_t(cnt) * row_bytes), "allocating fallback queries");
    SSG_CK(idx->fb_out.ensure(size_t(cnt) * k * 8), "allocating fallback results");
    int64_t *dlist = static_cast<int64_t *>(idx->fb_list.p);
    SSG_CK(cudaMemcpyAsync(dlist, list.data(), size_t(cnt) * 8, cudaMemcpyHostToDevice, idx->stream),
           "copying fallback list");
    SSG_CK(ssg::launch_gather_rows(dq, dlist, cnt, row_bytes, idx->fb_q.p, idx->stream, &idx->last_launches),
           "gathering fallback queries");
    uint32_t *fi = static_cast<uint32_t *>(idx->fb_out.p);
    float *fd = reinterpret_cast<float *>(fi + size_t(cnt) * k);
    const float *fqn = nullptr;
    if (idx->metric == SSG_METRIC_COSINE) {
        SSG_CK(idx->fb_qn.ensure(size_t(cnt) * 4), "allocating fallback query norms");
        SSG_CK(ssg::launch_row_norms(static_cast<const float *>(idx->fb_q.p), cnt, idx->dim,
                                     static_cast<float *>(idx->fb_qn.p), idx->stream, &idx->last_launches),
               "computing fallback query norms");
        fqn = static_cast<const float *>(idx->fb_qn.p);
    }
    // the scan timer reports the main scan only; the fallback shows in the call's time
    const int profile = idx->profile;
    idx->profile = 0;
    const int rc = run_exact_scan(idx, idx->fb_q.p, fqn, cnt, k, exclude_self, dlist, fi, fd, idx->fb_cand);
    idx->profile = profile;
    if (rc) return rc;
    SSG_CK(ssg::launch_scatter_results(fi, fd, dlist, cnt, k, d_ids, d_dists, idx->stream, &idx->last_launches),
           "scattering fallback results");
    SSG_CK(cudaStreamSynchronize(idx->stream), "running the fallback scan");
    return SSG_OK;
}

// ---------------------------------------------------------------------------
// The plain FP32 method on the tensor cores.  Every element is split into two
// BF16 pieces, x = hi + lo (+ a remainder below 2^-16 |x|); a tcgen05 scan
// over K = 3 kp with database rows laid out [lo | hi | hi] and query rows
// [hi | lo | hi] accumulates lo.hi + hi.lo + hi.hi in FP32, an approximation
// of x.q within c |x| |q|:
//   3.05 2^-16   the terms left out (lo.lo and both remainders);
//   2.2 kp 2^-23 FP32 accumulation: the 2 kp small products come first, so
//                their partial sums stay below 2^-7 |x||q|; the kp products
//                hi.hi then add at most 2^-23 of the largest magnitude in
//                the adder per product (17 terms per 16-product MMA), about
//                1.1 kp 2^-23 |x||q| in all, counted twice.
// The scan keeps kk = k + margin approximate candidates per query; the rerank
// computes their exact FP32 distances (the oracle's sequential sums) and
// certifies that no object outside the list can reach the result (rerank.cu,
// the completeness check); a query it cannot certify is recomputed by the
// exact direct scan, so the result is the plain method's, bit for bit.
// ---------------------------------------------------------------------------

// Candidates kept beyond the k + self needed by the plain method's scans:
// 0.45 k, at least 8, and for the squared distances at least dim / 12 (their
// error bound grows with dim times the squared norms, so wide vectors need a
// longer list to certify a query: at 768 dimensions and k = 10, 8 extra
// candidates left two thirds of C4's queries uncertified).
int plain_margin(const ssg_index *idx, int take) {
    if (idx->margin_param > 0) return idx->margin_param;
    int mg = std::max(8, (9 * take + 19) / 20);
    if (is_sq_metric(idx->metric)) mg = std::max<int>(mg, int(idx->dim / 12));
    return mg;
}

// How the plain method runs on the tensor cores: split K (0: it does not
// apply -- metric, dimension, or no scan kernel holds the tiles and the
// heaps), candidates kept per heap and candidates re-ranked per query.  The
// list is k + plain_margin long (a fallback costs far more than a longer
// list).  Each heap keeps the whole list when the one-CTA
// wide scan holds it with four ring stages or more.  Otherwise each of a
// query tile's two column heaps keeps part of it, as many as fit beside four
// ring stages and at least half the list: the completeness check then stops
// at the first full heap's last key, so the pair of heaps holds more than
// the list itself (about 2 x 32 for 33 neighbours on 96 dimensions, where
// 2 x 24 left 3.5 % of the queries uncertified).  The CTA-pair scan is the
// last resort.
struct PlainTcPlan {
    int k3 = 0, h = 0, rr = 0;
};
PlainTcPlan plain_tc_plan(const ssg_index *idx, int take) {
    const int metric = idx->metric;
    if (metric != SSG_METRIC_SQL2 && metric != SSG_METRIC_L2 && metric != SSG_METRIC_NORMCOSINE &&
        metric != SSG_METRIC_IP && metric != SSG_METRIC_COSINE)
        return {};
    const int k3 = 3 * ssg::tc_padded_k(idx->dim);
    if (k3 > 384) return {};
    const int margin = plain_margin(idx, take);
    const int kk = int(std::min<int64_t>(int64_t(take) + margin, idx->n));
    if (ssg::tc_wide_stages(k3, kk) >= 4) return {k3, kk, kk};
    int h = (kk + 1) / 2;
    if (ssg::tc_wide_stages(k3, h) >= 4) {
        while (h < kk && ssg::tc_wide_stages(k3, h + 1) >= 4) ++h;
        return {k3, h, 2 * h};
    }
    if (ssg::tc_wide_stages(k3, h) >= 3) return {k3, h, 2 * h};
    if (ssg::tc_pair_fits(k3, kk)) return {k3, kk, kk};
    return {};
}

// max |x|^2 over the database for the dot metrics' completeness check (the
// squared-distance metrics keep it current on every append).
int ensure_max_norm(ssg_index *idx) {
    if (is_sq_metric(idx->metric)) return SSG_OK;
    SSG_CK(idx->sq_norm.ensure(size_t(idx->n) * 4), "allocating squared norms");
    SSG_CK(idx->sq_max.ensure(16), "allocating the norm maximum");
    SSG_CK(cudaMemsetAsync(idx->sq_max.p, 0, 4, idx->stream), "clearing the norm maximum");
    SSG_CK(ssg::launch_row_sq_norms(static_cast<const float *>(idx->db.p), idx->n, idx->dim,
                                    static_cast<float *>(idx->sq_norm.p), static_cast<float *>(idx->sq_max.p),
                                    idx->stream, &idx->last_launches),
           "computing squared norms");
    SSG_CK(cudaMemcpyAsync(&idx->max_x_sq, idx->sq_max.p, 4, cudaMemcpyDeviceToHost, idx->stream),
           "reading the norm maximum");
    SSG_CK(cudaStreamSynchronize(idx->stream), "computing squared norms");
    return SSG_OK;
}

// Two-piece tiles of the database (database role; the query role as well for
// allknn), |x|^2 per padded row, and max |x|^2 for the dot metrics' check.
int ensure_plain_tiles(ssg_index *idx, bool query_role) {
    const int64_t tiles = (ssg::tc_tiles(idx->n) + 1) / 2 * 2;
    const size_t tb = ssg::tc_tile_bytes(3 * ssg::tc_padded_k(idx->dim));
    const float *x = static_cast<const float *>(idx->db.p);
    if (idx->ps_rows != idx->n) {
        idx->ps_qrows = -1;
        SSG_CK(idx->ps_db.ensure(size_t(tiles) * tb), "allocating split database tiles");
        SSG_CK(ssg::launch_bf16_tiles(x, idx->n, idx->dim, tiles, static_cast<uint8_t *>(idx->ps_db.p), idx->stream,
                                      &idx->last_launches, nullptr, 1),
               "building split database tiles");
        SSG_CK(idx->ps_norm.ensure(size_t(tiles) * 128 * 4), "allocating split tile norms");
        // |x|^2 per row for the squared-distance and dot keys, 1 / |x| for Cosine's
        SSG_CK(ssg::launch_tc_norms(idx->metric == SSG_METRIC_COSINE ? SSG_METRIC_COSINE : SSG_METRIC_SQL2, x,
                                    idx->n, idx->dim, tiles * 128,
                                    static_cast<float *>(idx->ps_norm.p), idx->stream, &idx->last_launches),
               "computing split tile norms");
        SSG_RC(ensure_max_norm(idx));
        SSG_CK(cudaStreamSynchronize(idx->stream), "building split database tiles");
        idx->ps_rows = idx->n;
    }
    if (query_role && idx->ps_qrows != idx->n) {
        SSG_CK(idx->ps_dbq.ensure(size_t(tiles) * tb), "allocating split query-role tiles");
        SSG_CK(ssg::launch_bf16_tiles(x, idx->n, idx->dim, tiles, static_cast<uint8_t *>(idx->ps_dbq.p),
                                      idx->stream, &idx->last_launches, nullptr, 2),
               "building split query-role tiles");
        idx->ps_qrows = idx->n;
    }
    return SSG_OK;
}

// allknn's locality order needs at least this many rows (below it the order's
// set-up would cost more than the heap insertions it saves)
constexpr int64_t kLocalityMinRows = 32768;

int ensure_plain_locality(ssg_index *idx);

int run_plain_tc(ssg_index *idx, const float *dq, const float *dqn, int64_t m, int k, int exclude_self,
                 uint32_t *d_ids, float *d_dists, bool queries_are_db, const PlainTcPlan &plan) {
    const int kk = plan.h, k3 = plan.k3;
    const bool sq = is_sq_metric(idx->metric);
    const int kp = ssg::tc_padded_k(idx->dim);
    SSG_RC(ensure_plain_tiles(idx, queries_are_db));
    const int64_t qctas = (m + 127) / 128;
    const int64_t n_tiles = ssg::tc_tiles(idx->n);
    int64_t splits = idx->splits_param > 0 ? idx->splits_param : wave_splits(qctas, ssg::device_sm_count(), n_tiles);
    splits = std::max<int64_t>(1, std::min<int64_t>(splits, n_tiles));
    const int segs = int(splits) * ssg::tc_segments_per_split(1);
    const size_t per_query = size_t(segs) * kk * 8;
    int64_t chunk = std::max<int64_t>(256, int64_t((size_t(1) << 30) / per_query) / 256 * 256);
    chunk = std::min<int64_t>(chunk, qctas * 128);
    SSG_CK(idx->cand.ensure(per_query * size_t(chunk)), "allocating candidate scratch");
    SSG_CK(idx->status.ensure(sizeof(int)), "allocating the status word");
    SSG_CK(cudaMemsetAsync(idx->status.p, 0, sizeof(int), idx->stream), "clearing the status word");
    SSG_CK(idx->flags.ensure(size_t(m) * 4 + 16), "allocating query flags");
    SSG_CK(cudaMemsetAsync(idx->flags.p, 0, size_t(m) * 4 + 16, idx->stream), "clearing query flags");
    SSG_CK(idx->qsq.ensure(size_t(chunk) * 4 + 16), "allocating query norms");
    const size_t tb = ssg::tc_tile_bytes(k3);
    const uint8_t *qtiles = static_cast<const uint8_t *>(idx->ps_dbq.p);
    if (!queries_are_db) {
        const int64_t qt_alloc = (qctas + 1) / 2 * 2;  // even: the pair scan reads query tiles in pairs
        SSG_CK(idx->ps_q.ensure(size_t(qt_alloc) * tb), "allocating split query tiles");
        SSG_CK(ssg::launch_bf16_tiles(dq, m, idx->dim, qt_alloc, static_cast<uint8_t *>(idx->ps_q.p), idx->stream,
                                      &idx->last_launches, nullptr, 2),
               "building split query tiles");
        qtiles = static_cast<const uint8_t *>(idx->ps_q.p);
    }
    // allknn in one launch: the database in its locality order (rows grouped
    // by nearest pivot, each query tile starting at its own group), so the
    // heaps hold near neighbours from the first tiles on and few later
    // columns pass their bound
    const uint8_t *dtiles = static_cast<const uint8_t *>(idx->ps_db.p);
    const float *dnorm = static_cast<const float *>(idx->ps_norm.p);
    const uint32_t *perm = nullptr;
    const int *rot = nullptr;
    if (queries_are_db && idx->locality_param && m == idx->n && idx->n >= kLocalityMinRows && chunk >= m) {
        SSG_RC(ensure_plain_locality(idx));
        qtiles = static_cast<const uint8_t *>(idx->loc_ps_dbq.p);
        dtiles = static_cast<const uint8_t *>(idx->loc_ps_db.p);
        dnorm = static_cast<const float *>(idx->loc_ps_norm.p);
        perm = static_cast<const uint32_t *>(idx->loc_perm.p);
        rot = static_cast<const int *>(idx->loc_rot.p);
    }
    // every heap of a query -- its splits and the two column heaps of each
    // CTA -- shares one bound (all ones: none yet)
    uint32_t *qbound = nullptr;
    if (segs > 1) {
        SSG_CK(idx->qbound.ensure(size_t(chunk) * 4), "allocating query bounds");
        qbound = static_cast<uint32_t *>(idx->qbound.p);
    }
    // |a - a_exact| <= c |x| |q| (see above) plus the exact evaluation's own
    // error: (d + 2) 2^-24 |x| |q| for a dot product; the squared-distance
    // metrics add c |x| |q| <= c/2 (|x| + |q|)^2 to the GEMM-form allowance
    // 4 (d + 2) 2^-24 (|x| + |q|)^2
    const float c = 3.05f * 1.52587890625e-5f + 2.2f * float(kp) * 1.1920929e-7f;
    const float ulp24 = 5.9604645e-8f;
    int *flags = static_cast<int *>(idx->flags.p);
    int *flag_count = flags + m;
    float *qsq = static_cast<float *>(idx->qsq.p);
    ScanTimer timer(idx);
    for (int64_t c0 = 0; c0 < m; c0 += chunk) {
        const int64_t mc = std::min<int64_t>(chunk, m - c0);
        if (qbound) SSG_CK(cudaMemsetAsync(qbound, 0xff, size_t(mc) * 4, idx->stream), "clearing query bounds");
        SSG_RC(timer.begin());
        SSG_CK(ssg::launch_tc_scan(idx->metric, qtiles + size_t(c0 / 128) * tb, dtiles, dnorm, idx->n, mc, k3, kk,
                                   int(splits), static_cast<uint64_t *>(idx->cand.p),
                                   static_cast<int *>(idx->status.p), idx->stream, &idx->last_launches, nullptr, perm,
                                   rot, true, idx->wave_param, idx->pair_param != 0, qbound),
               "launching the split tensor-core scan");
        SSG_RC(timer.end());
        const float *qc = dq + size_t(c0) * idx->dim;
        SSG_CK(ssg::launch_row_sq_norms(qc, mc, idx->dim, qsq, qsq + chunk, idx->stream, &idx->last_launches),
               "computing query norms");
        ssg::FinalizeArgs f{};
        SSG_RC(reduce_segments(idx, static_cast<const uint64_t *>(idx->cand.p), mc, segs, kk, &f.cand, &f.segs));
        f.kk = kk;
        f.m = mc;
        f.k_out = k;
        f.exclude_self = exclude_self;
        f.self_base = c0;
        f.out_ids = d_ids + size_t(c0) * k;
        f.out_dists = d_dists + size_t(c0) * k;
        f.n_rows = idx->n;
        f.rerank = std::min(plan.rr, f.segs * kk);
        f.check = sq ? 1 : (idx->metric == SSG_METRIC_COSINE ? 3 : 2);
        f.q_sq = qsq;
        f.max_x_sq = idx->max_x_sq;
        f.err_scale = sq ? 4.0f * float(idx->dim + 2) * ulp24 + 0.5f * c
                         : (f.check == 3 ? c + float(2 * idx->dim + 16) * ulp24 : c + float(idx->dim + 2) * ulp24);
        f.n_total = idx->n;
        f.flags = flags + c0;
        f.flag_count = flag_count;
        SSG_CK(ssg::launch_finalize_rerank(idx->metric, f, static_cast<const float *>(idx->db.p),
                                           static_cast<const float *>(idx->db_norm.p), idx->dim, qc,
                                           dqn ? dqn + c0 : nullptr,
                                           idx->stream, &idx->last_launches),
               "launching the rerank kernel");
        SSG_RC(timer.collect());
    }
    int status = 0, nflag = 0;
    SSG_CK(cudaMemcpyAsync(&status, idx->status.p, sizeof(int), cudaMemcpyDeviceToHost, idx->stream),
           "reading the status word");
    SSG_CK(cudaMemcpyAsync(&nflag, flag_count, sizeof(int), cudaMemcpyDeviceToHost, idx->stream), "reading flags");
    SSG_CK(cudaStreamSynchronize(idx->stream), "running the split tensor-core scan");
    if (status != 0)
        return fail(idx, SSG_ETIMEOUT, "a bounded wait in the split tensor-core scan gave up (code %d)", status);
    idx->last_fallbacks = nflag;
    return run_fallback(idx, dq, m, k, exclude_self, flags, nflag, d_ids, d_dists);
}

// The plain method on the tensor cores for wide vectors (dim > 128, where a
// resident split query tile does not fit): the same two-piece split and
// certificate through the K-streaming scan, both operands streamed along
// K = 3 kp (kp = dim padded to 64).  Returns SSG_OK, an error, or
// kPlainNotApplicable when the list does not fit the scan's heaps.
constexpr int kPlainNotApplicable = 1;

int ensure_plain_stream_tiles(ssg_index *idx, bool query_role) {
    const int64_t tiles = ssg::tc_tiles(idx->n);
    const float *x = static_cast<const float *>(idx->db.p);
    const size_t tb = 3 * ssg::stream_tile_bytes(idx->dim, 0);
    if (idx->pss_rows != idx->n) {
        idx->pss_qrows = -1;
        SSG_CK(idx->pss_db.ensure(size_t(tiles) * tb), "allocating split database tiles");
        SSG_CK(ssg::launch_stream_tiles(x, idx->n, idx->dim, 0, tiles, static_cast<uint8_t *>(idx->pss_db.p),
                                        nullptr, idx->stream, &idx->last_launches, 1),
               "building split database tiles");
        SSG_CK(idx->pss_alpha.ensure(size_t(tiles) * 128 * 4), "allocating epilogue coefficients");
        SSG_CK(idx->pss_beta.ensure(size_t(tiles) * 128 * 4), "allocating epilogue coefficients");
        SSG_CK(ssg::launch_stream_coefs(idx->metric, x, idx->n, idx->dim, tiles * 128, nullptr,
                                        static_cast<float *>(idx->pss_alpha.p), static_cast<float *>(idx->pss_beta.p),
                                        idx->stream, &idx->last_launches),
               "computing epilogue coefficients");
        SSG_RC(ensure_max_norm(idx));
        SSG_CK(cudaStreamSynchronize(idx->stream), "building split database tiles");
        idx->pss_rows = idx->n;
    }
    if (query_role && idx->pss_qrows != idx->n) {
        SSG_CK(idx->pss_dbq.ensure(size_t(tiles) * tb), "allocating split query-role tiles");
        SSG_CK(ssg::launch_stream_tiles(x, idx->n, idx->dim, 0, tiles, static_cast<uint8_t *>(idx->pss_dbq.p),
                                        nullptr, idx->stream, &idx->last_launches, 2),
               "building split query-role tiles");
        idx->pss_qrows = idx->n;
    }
    return SSG_OK;
}

int run_plain_stream(ssg_index *idx, const float *dq, const float *dqn, int64_t m, int k, int exclude_self,
                     uint32_t *d_ids, float *d_dists, bool queries_are_db) {
    const int metric = idx->metric;
    if (metric != SSG_METRIC_SQL2 && metric != SSG_METRIC_L2 && metric != SSG_METRIC_NORMCOSINE &&
        metric != SSG_METRIC_IP && metric != SSG_METRIC_COSINE)
        return kPlainNotApplicable;
    const bool sq = is_sq_metric(metric);
    const int take = k + (exclude_self ? 1 : 0);
    // the margin shrinks (down to the list's basic 0.45 k) until the scan's heaps hold it
    const int margin = plain_margin(idx, take);
    const int base = std::min(margin, std::max(8, (9 * take + 19) / 20));
    int kk = int(std::min<int64_t>(int64_t(take) + margin, idx->n));
    const int kk_min = int(std::min<int64_t>(int64_t(take) + base, idx->n));
    const int heap_rows = ssg::stream_heap_rows(m);
    int cs = 0, stages = 0;
    while (kk > kk_min && !ssg::stream_choose(kk, heap_rows, &cs, &stages)) --kk;
    if (!ssg::stream_choose(kk, heap_rows, &cs, &stages)) return kPlainNotApplicable;
    const int kp = ssg::stream_kbytes(idx->dim, 0) / 2;  // elements per piece
    const int64_t k3 = 3 * int64_t(kp);
    SSG_RC(ensure_plain_stream_tiles(idx, queries_are_db));
    const int64_t qtiles = (m + 127) / 128;
    const int64_t n_tiles = ssg::tc_tiles(idx->n);
    int64_t splits = idx->splits_param > 0 ? idx->splits_param : wave_splits(qtiles, ssg::device_sm_count(), n_tiles);
    splits = std::max<int64_t>(1, std::min<int64_t>(splits, n_tiles));
    const int segs = int(splits) * cs;
    const size_t per_query = size_t(segs) * kk * 8;
    int64_t chunk = std::max<int64_t>(128, int64_t((size_t(1) << 30) / per_query) / 128 * 128);
    chunk = std::min<int64_t>(chunk, qtiles * 128);
    SSG_CK(idx->cand.ensure(per_query * size_t(chunk)), "allocating candidate scratch");
    SSG_CK(idx->status.ensure(sizeof(int)), "allocating the status word");
    SSG_CK(cudaMemsetAsync(idx->status.p, 0, sizeof(int), idx->stream), "clearing the status word");
    SSG_CK(idx->flags.ensure(size_t(m) * 4 + 16), "allocating query flags");
    SSG_CK(cudaMemsetAsync(idx->flags.p, 0, size_t(m) * 4 + 16, idx->stream), "clearing query flags");
    SSG_CK(idx->qsq.ensure(size_t(chunk) * 4 + 16), "allocating query norms");
    const size_t tb = 3 * ssg::stream_tile_bytes(idx->dim, 0);
    const uint8_t *qt = static_cast<const uint8_t *>(idx->pss_dbq.p);
    if (!queries_are_db) {
        SSG_CK(idx->pss_q.ensure(size_t(qtiles) * tb), "allocating split query tiles");
        SSG_CK(ssg::launch_stream_tiles(dq, m, idx->dim, 0, qtiles, static_cast<uint8_t *>(idx->pss_q.p), nullptr,
                                        idx->stream, &idx->last_launches, 2),
               "building split query tiles");
        qt = static_cast<const uint8_t *>(idx->pss_q.p);
    }
    // the K-streaming scan's shared pruning bounds, as for its reduced-precision use
    uint32_t *gbound = nullptr;
    if (kk >= 32 && 2 * splits * cs >= kk) {
        SSG_CK(idx->gbound.ensure(size_t(chunk) * ssg::kBoundWords * 4), "allocating query bounds");
        gbound = static_cast<uint32_t *>(idx->gbound.p);
    }
    // the error bound of the split (run_plain_tc) with this kp
    const float c = 3.05f * 1.52587890625e-5f + 2.2f * float(kp) * 1.1920929e-7f;
    const float ulp24 = 5.9604645e-8f;
    int *flags = static_cast<int *>(idx->flags.p);
    int *flag_count = flags + m;
    float *qsq = static_cast<float *>(idx->qsq.p);
    ScanTimer timer(idx);
    for (int64_t c0 = 0; c0 < m; c0 += chunk) {
        const int64_t mc = std::min<int64_t>(chunk, m - c0);
        if (gbound)
            SSG_CK(cudaMemsetAsync(gbound, 0, size_t(mc) * ssg::kBoundWords * 4, idx->stream),
                   "clearing query bounds");
        SSG_RC(timer.begin());
        SSG_CK(ssg::launch_stream_scan(qt + size_t(c0 / 128) * tb, static_cast<const uint8_t *>(idx->pss_db.p),
                                       static_cast<const float *>(idx->pss_alpha.p),
                                       static_cast<const float *>(idx->pss_beta.p), nullptr, idx->n, mc, k3, 0, kk,
                                       int(splits), heap_rows, gbound, static_cast<uint64_t *>(idx->cand.p),
                                       static_cast<int *>(idx->status.p), idx->stream, &idx->last_launches, nullptr),
               "launching the split streaming scan");
        SSG_RC(timer.end());
        const float *qc = dq + size_t(c0) * idx->dim;
        SSG_CK(ssg::launch_row_sq_norms(qc, mc, idx->dim, qsq, qsq + chunk, idx->stream, &idx->last_launches),
               "computing query norms");
        ssg::FinalizeArgs f{};
        SSG_RC(reduce_segments(idx, static_cast<const uint64_t *>(idx->cand.p), mc, segs, kk, &f.cand, &f.segs));
        f.kk = kk;
        f.m = mc;
        f.k_out = k;
        f.exclude_self = exclude_self;
        f.self_base = c0;
        f.out_ids = d_ids + size_t(c0) * k;
        f.out_dists = d_dists + size_t(c0) * k;
        f.n_rows = idx->n;
        f.check = sq ? 1 : (idx->metric == SSG_METRIC_COSINE ? 3 : 2);
        f.q_sq = qsq;
        f.max_x_sq = idx->max_x_sq;
        f.err_scale = sq ? 4.0f * float(idx->dim + 2) * ulp24 + 0.5f * c
                         : (f.check == 3 ? c + float(2 * idx->dim + 16) * ulp24 : c + float(idx->dim + 2) * ulp24);
        f.n_total = idx->n;
        f.flags = flags + c0;
        f.flag_count = flag_count;
        SSG_CK(ssg::launch_finalize_rerank(idx->metric, f, static_cast<const float *>(idx->db.p),
                                           static_cast<const float *>(idx->db_norm.p), idx->dim, qc,
                                           dqn ? dqn + c0 : nullptr,
                                           idx->stream, &idx->last_launches),
               "launching the rerank kernel");
        SSG_RC(timer.collect());
    }
    int status = 0, nflag = 0;
    SSG_CK(cudaMemcpyAsync(&status, idx->status.p, sizeof(int), cudaMemcpyDeviceToHost, idx->stream),
           "reading the status word");
    SSG_CK(cudaMemcpyAsync(&nflag, flag_count, sizeof(int), cudaMemcpyDeviceToHost, idx->stream), "reading flags");
    SSG_CK(cudaStreamSynchronize(idx->stream), "running the split streaming scan");
    if (status != 0)
        return fail(idx, SSG_ETIMEOUT, "a bounded wait in the split streaming scan gave up (code %d)", status);
    idx->last_fallbacks = nflag;
    return run_fallback(idx, dq, m, k, exclude_self, flags, nflag, d_ids, d_dists);
}

int run_knn_tc(ssg_index *idx, const void *dq, const float *dqn, int64_t m, int k, int exclude_self,
               uint32_t *d_ids, float *d_dists, bool queries_are_db);
int run_knn_stream(ssg_index *idx, const void *dq, const float *dqn, int64_t m, int k, int exclude_self,
                   uint32_t *d_ids, float *d_dists, bool queries_are_db);

// Frees the plain method's split tiles (and their locality-ordered copies).
void release_plain_tiles(ssg_index *idx) {
    for (DevBuf *b : {&idx->ps_db, &idx->ps_dbq, &idx->ps_norm, &idx->ps_q, &idx->pss_db, &idx->pss_dbq,
                      &idx->pss_alpha, &idx->pss_beta, &idx->pss_q, &idx->loc_ps_db, &idx->loc_ps_dbq,
                      &idx->loc_ps_norm})
        b->release();
    idx->ps_rows = idx->ps_qrows = idx->pss_rows = idx->pss_qrows = idx->loc_ps_n = -1;
}

// Databases below this many rows keep the plain method on the CUDA cores
// (the split tiles would cost more than the scan they speed up).
constexpr int64_t kPlainTcMinRows = 4096;

// Dispatch: BF16 tensor-core mode, Hamming, or the plain FP32 method (on the
// tensor cores in split form where it applies, else GEMM form when its heaps
// fit, otherwise the exact direct scan).
int run_knn(ssg_index *idx, const void *dq, const float *dqn, int64_t m, int k, int exclude_self,
            uint32_t *d_ids, float *d_dists, bool queries_are_db = false) {
    if (idx->prec != SSG_PREC_FP32 && !idx->plain_param) {
        if (uses_stream(idx)) return run_knn_stream(idx, dq, dqn, m, k, exclude_self, d_ids, d_dists, queries_are_db);
        return run_knn_tc(idx, dq, dqn, m, k, exclude_self, d_ids, d_dists, queries_are_db);
    }
    idx->last_fallbacks = 0;
    idx->last_plain_tc = 0;
    if (idx->metric != SSG_METRIC_HAMMING && !idx->exact_scan_param && idx->plain_tc_param &&
        idx->n >= kPlainTcMinRows && !idx->capturing) {
        // the split tiles take 1.5x the FP32 database per role: when device
        // memory runs out the CUDA-core form answers instead (it rewrites
        // every output row)
        const PlainTcPlan plan = plain_tc_plan(idx, k + (exclude_self ? 1 : 0));
        int rc = kPlainNotApplicable;
        if (plan.k3 > 0)
            rc = run_plain_tc(idx, static_cast<const float *>(dq), dqn, m, k, exclude_self, d_ids, d_dists,
                              queries_are_db, plan);
        else if (ssg::tc_padded_k(idx->dim) > 128)
            rc = run_plain_stream(idx, static_cast<const float *>(dq), dqn, m, k, exclude_self, d_ids, d_dists,
                                  queries_are_db);
        if (rc == SSG_ENOMEM) release_plain_tiles(idx);
        else if (rc != kPlainNotApplicable) {
            idx->last_plain_tc = 1;
            return rc;
        }
    }
    if (idx->metric != SSG_METRIC_HAMMING && !idx->exact_scan_param) {
        const int take = k + (exclude_self ? 1 : 0);
        int64_t kk = is_sq_metric(idx->metric) ? int64_t(take) + gemm_margin(idx, take) : take;
        // the longer list of the tensor-core forms where the heaps hold it
        if (is_sq_metric(idx->metric) && ssg::gemm_fits(int(take + plain_margin(idx, take))))
            kk = int64_t(take) + plain_margin(idx, take);
        kk = std::min<int64_t>(kk, std::max<int64_t>(1, idx->n));
        if (ssg::gemm_fits(int(kk)))
            return run_gemm(idx, static_cast<const float *>(dq), dqn, m, k, exclude_self, d_ids, d_dists, int(kk));
    }
    return run_exact_scan(idx, dq, dqn, m, k, exclude_self, nullptr, d_ids, d_dists, idx->cand);
}

// The BF16 pipeline: operand tiles of the queries (or the database itself for
// allknn), the tcgen05 scan keeping kk = overfetch * k approximate candidates
// per query and split, then the exact FP32 rerank + (distance, id) merge.
int run_knn_tc_filter(ssg_index *idx, const void *dq, const float *dqn, int64_t m, int k, int exclude_self,
                      uint32_t *d_ids, float *d_dists, bool queries_are_db, int kk);

// Candidates kept per query by the reduced-precision scans for `take`
// neighbours: the over-fetch, at least take, at most max(take, min(n, 4096)).
int64_t overfetch_kk(const ssg_index *idx, int take) {
    int64_t kk64 = int64_t(idx->overfetch * take + 0.999);
    kk64 = std::max<int64_t>(kk64, take);
    return std::min<int64_t>(kk64, std::max<int64_t>(take, std::min<int64_t>(idx->n, 4096)));
}

// The pivots' chain order: rank[p] = place of pivot p in a greedy chain
// that starts at pivot 0 and always links the nearest pivot not yet linked
// among the last link's kNear nearest pivots (a BF16 scan of the pivots
// against themselves), else among the lists of the links before it, else the
// lowest-numbered pivot left.  Pivots near each other so take nearby places,
// and the groups of one dense region of the data sit side by side.  Leaves
// rank empty when the pivots' scan does not fit (the groups then keep pivot
// order).
int pivot_chain(ssg_index *idx, const uint32_t *pmap, int P, DevBuf &rank) {
    constexpr int kNear = 16;
    const int kk = std::min(kNear + 1, P);  // the pivot itself comes first
    const int64_t tiles = (ssg::tc_tiles(P) + 1) / 2 * 2;
    const float *x = static_cast<const float *>(idx->db.p);
    DevBuf t, nrm, keys;
    SSG_CK(t.ensure(size_t(tiles) * ssg::tc_tile_bytes(idx->dim)), "allocating pivot tiles");
    SSG_CK(nrm.ensure(size_t(tiles) * 128 * 4), "allocating pivot norms");
    SSG_CK(ssg::launch_bf16_tiles(x, P, idx->dim, tiles, static_cast<uint8_t *>(t.p), idx->stream,
                                  &idx->last_launches, pmap, 0),
           "building pivot tiles");
    SSG_CK(ssg::launch_tc_norms(idx->metric, x, P, idx->dim, tiles * 128, static_cast<float *>(nrm.p), idx->stream,
                                &idx->last_launches, pmap),
           "computing pivot norms");
    const int max_segs = std::max(ssg::tc_segments_per_split(1), ssg::tc_segments_per_split(2));
    SSG_CK(keys.ensure(size_t(P) * max_segs * kk * 8), "allocating pivot neighbour lists");
    SSG_CK(cudaMemsetAsync(idx->status.p, 0, sizeof(int), idx->stream), "clearing the status word");
    int qt = 1;
    const cudaError_t e = ssg::launch_tc_scan(idx->metric, static_cast<const uint8_t *>(t.p),
                                              static_cast<const uint8_t *>(t.p), static_cast<const float *>(nrm.p), P, P,
                                              idx->dim, kk, 1, static_cast<uint64_t *>(keys.p),
                                              static_cast<int *>(idx->status.p), idx->stream, &idx->last_launches, &qt,
                                              nullptr, nullptr, true);
    if (e == cudaErrorInvalidValue) return SSG_OK;  // no tile shape fits (nothing launched): pivot order
    SSG_CK(e, "launching the pivots' scan");
    const int segs = ssg::tc_segments_per_split(qt);
    std::vector<uint64_t> h(size_t(P) * segs * kk);
    int status = 0;
    SSG_CK(cudaMemcpyAsync(h.data(), keys.p, h.size() * 8, cudaMemcpyDeviceToHost, idx->stream),
           "reading pivot neighbour lists");
    SSG_CK(cudaMemcpyAsync(&status, idx->status.p, sizeof(int), cudaMemcpyDeviceToHost, idx->stream),
           "reading the status word");
    SSG_CK(cudaStreamSynchronize(idx->stream), "scanning the pivots");
    if (status != 0)
        return fail(idx, SSG_ETIMEOUT, "a bounded wait in the pivots' scan gave up (code %d)", status);
    // each pivot's nearest other pivots, nearest first
    std::vector<uint32_t> near(size_t(P) * kNear, UINT32_MAX);
    std::vector<uint64_t> row(size_t(segs) * kk);
    for (int p = 0; p < P; ++p) {
        std::copy(h.begin() + size_t(p) * row.size(), h.begin() + size_t(p + 1) * row.size(), row.begin());
        std::sort(row.begin(), row.end());
        int c = 0;
        for (size_t i = 0; i < row.size() && c < kNear; ++i) {
            if (row[i] == ssg::KEY_EMPTY) break;
            const uint32_t q = ssg::key_id0(row[i]);
            if (q == uint32_t(p) || q >= uint32_t(P)) continue;
            near[size_t(p) * kNear + c++] = q;
        }
    }
    // the last link's list, then those of up to 64 links before it
    std::vector<uint32_t> place(static_cast<size_t>(P));
    ssg::greedy_chain(near.data(), P, kNear, 64, place.data());
    SSG_CK(rank.ensure(size_t(P) * 4), "allocating pivot ranks");
    SSG_CK(cudaMemcpyAsync(rank.p, place.data(), size_t(P) * 4, cudaMemcpyHostToDevice, idx->stream),
           "copying pivot ranks");
    SSG_CK(cudaStreamSynchronize(idx->stream), "copying pivot ranks");
    return SSG_OK;
}

// Builds allknn's locality order (tc_bf16.cu, launch_locality_order): P
// evenly spaced rows as pivots (one per loc_rows_param rows), each row's
// nearest pivot by a kk = 1 scan of the database's tiles in the query role
// (`qtiles`: the BF16 tiles, or the plain method's split tiles with `split`
// 2) against the pivots' tiles, rows grouped by pivot, the groups in the
// pivots' chain order (pivot_chain); position -> id in loc_perm and each
// query tile's start tile in loc_rot.  The order only groups rows: any
// assignment to pivots and any group order give the same results.  Kept
// until the database or the parameters change.
int ensure_locality_order(ssg_index *idx, const uint8_t *qtiles, int split) {
    if (idx->loc_n == idx->n) return SSG_OK;
    const int64_t n = idx->n;
    const int64_t per = idx->loc_rows_param;
    const int P = int(std::min<int64_t>(16384, std::max<int64_t>(128, (n / per + 127) / 128 * 128)));
    std::vector<uint32_t> prow(static_cast<size_t>(P));
    for (int i = 0; i < P; ++i) prow[size_t(i)] = uint32_t(int64_t(i) * n / P);
    const int64_t kdim = split ? 3 * ssg::tc_padded_k(idx->dim) : idx->dim;
    const size_t tb = ssg::tc_tile_bytes(kdim);
    const int64_t ptiles = (ssg::tc_tiles(P) + 1) / 2 * 2;
    const int segs = ssg::tc_segments_per_split(1);
    DevBuf prow_d, pt, pn, work;
    SSG_CK(prow_d.ensure(size_t(P) * 4), "allocating the pivot list");
    SSG_CK(cudaMemcpyAsync(prow_d.p, prow.data(), size_t(P) * 4, cudaMemcpyHostToDevice, idx->stream),
           "copying the pivot list");
    SSG_CK(pt.ensure(size_t(ptiles) * tb), "allocating pivot tiles");
    SSG_CK(pn.ensure(size_t(ptiles) * 128 * 4), "allocating pivot norms");
    const float *x = static_cast<const float *>(idx->db.p);
    const uint32_t *pmap = static_cast<const uint32_t *>(prow_d.p);
    SSG_CK(ssg::launch_bf16_tiles(x, P, idx->dim, ptiles, static_cast<uint8_t *>(pt.p), idx->stream,
                                  &idx->last_launches, pmap, split ? 1 : 0),
           "building pivot tiles");
    SSG_CK(ssg::launch_tc_norms(idx->metric, x, P, idx->dim, ptiles * 128, static_cast<float *>(pn.p), idx->stream,
                                &idx->last_launches, pmap),
           "computing pivot norms");
    SSG_CK(idx->status.ensure(sizeof(int)), "allocating the status word");
    DevBuf rank;
    if (idx->loc_chain_param) SSG_RC(pivot_chain(idx, pmap, P, rank));
    // nearest pivot of every row (its keys), then per-row pivot, bucket
    // counts, starts and cursors in one scratch buffer
    const size_t cand_bytes = size_t(n) * segs * 8;
    SSG_CK(work.ensure(cand_bytes + size_t(n) * 4 + size_t(P) * 12), "allocating locality scratch");
    uint64_t *cand = static_cast<uint64_t *>(work.p);
    uint32_t *pivot = reinterpret_cast<uint32_t *>(static_cast<char *>(work.p) + cand_bytes);
    int *count = reinterpret_cast<int *>(pivot + n);
    SSG_CK(cudaMemsetAsync(idx->status.p, 0, sizeof(int), idx->stream), "clearing the status word");
    // the split tiles' K only fits the wide scan
    SSG_CK(ssg::launch_tc_scan(idx->metric, qtiles, static_cast<const uint8_t *>(pt.p),
                               static_cast<const float *>(pn.p), P, n, kdim, 1, 1, cand,
                               static_cast<int *>(idx->status.p), idx->stream, &idx->last_launches, nullptr, nullptr,
                               nullptr, split != 0),
           "launching the pivot scan");
    const int64_t qtiles_n = ssg::tc_tiles(n);
    SSG_CK(idx->loc_perm.ensure(size_t(n) * 4), "allocating the locality order");
    SSG_CK(idx->loc_rot.ensure(size_t(qtiles_n) * 4), "allocating scan start tiles");
    SSG_CK(ssg::launch_locality_order(cand, n, segs, P, static_cast<const uint32_t *>(rank.p), pivot, count,
                                      count + P, count + 2 * P, static_cast<uint32_t *>(idx->loc_perm.p),
                                      static_cast<int *>(idx->loc_rot.p), idx->stream, &idx->last_launches),
           "ordering rows by pivot");
    int status = 0;
    SSG_CK(cudaMemcpyAsync(&status, idx->status.p, sizeof(int), cudaMemcpyDeviceToHost, idx->stream),
           "reading the status word");
    SSG_CK(cudaStreamSynchronize(idx->stream), "building the locality order");
    if (status != 0)
        return fail(idx, SSG_ETIMEOUT, "a bounded wait in the pivot scan gave up (code %d)", status);
    idx->loc_n = n;
    return SSG_OK;
}

// The BF16 tiles and norms in the locality order (built from the BF16 tiles'
// pivot scan when no order exists yet).
int ensure_locality(ssg_index *idx) {
    if (idx->loc_n == idx->n && idx->loc_tiles.p && idx->loc_norm.p && idx->loc_bf16_n == idx->n) return SSG_OK;
    SSG_RC(ensure_locality_order(idx, static_cast<const uint8_t *>(idx->tc_db.p), 0));
    const int64_t n = idx->n;
    const float *x = static_cast<const float *>(idx->db.p);
    const uint32_t *perm = static_cast<const uint32_t *>(idx->loc_perm.p);
    const int64_t tiles = (ssg::tc_tiles(n) + 1) / 2 * 2;
    SSG_CK(idx->loc_tiles.ensure(size_t(tiles) * ssg::tc_tile_bytes(idx->dim)), "allocating locality-ordered tiles");
    SSG_CK(ssg::launch_bf16_tiles(x, n, idx->dim, tiles, static_cast<uint8_t *>(idx->loc_tiles.p), idx->stream,
                                  &idx->last_launches, perm),
           "building locality-ordered tiles");
    SSG_CK(idx->loc_norm.ensure(size_t(tiles) * 128 * 4), "allocating locality-ordered norms");
    SSG_CK(ssg::launch_tc_norms(idx->metric, x, n, idx->dim, tiles * 128, static_cast<float *>(idx->loc_norm.p),
                                idx->stream, &idx->last_launches, perm),
           "computing locality-ordered norms");
    SSG_CK(cudaStreamSynchronize(idx->stream), "building locality-ordered tiles");
    idx->loc_bf16_n = n;
    return SSG_OK;
}

// The plain method's split tiles (database and query roles) and |x|^2 in the
// locality order, from a pivot scan of the split tiles.
int ensure_plain_locality(ssg_index *idx) {
    if (idx->loc_ps_n == idx->n && idx->loc_n == idx->n) return SSG_OK;
    SSG_RC(ensure_locality_order(idx, static_cast<const uint8_t *>(idx->ps_dbq.p), 2));
    const int64_t n = idx->n;
    const float *x = static_cast<const float *>(idx->db.p);
    const uint32_t *perm = static_cast<const uint32_t *>(idx->loc_perm.p);
    const int64_t tiles = (ssg::tc_tiles(n) + 1) / 2 * 2;
    const size_t tb = ssg::tc_tile_bytes(3 * ssg::tc_padded_k(idx->dim));
    SSG_CK(idx->loc_ps_db.ensure(size_t(tiles) * tb), "allocating locality-ordered split tiles");
    SSG_CK(ssg::launch_bf16_tiles(x, n, idx->dim, tiles, static_cast<uint8_t *>(idx->loc_ps_db.p), idx->stream,
                                  &idx->last_launches, perm, 1),
           "building locality-ordered split tiles");
    SSG_CK(idx->loc_ps_dbq.ensure(size_t(tiles) * tb), "allocating locality-ordered split query tiles");
    SSG_CK(ssg::launch_bf16_tiles(x, n, idx->dim, tiles, static_cast<uint8_t *>(idx->loc_ps_dbq.p), idx->stream,
                                  &idx->last_launches, perm, 2),
           "building locality-ordered split query tiles");
    SSG_CK(idx->loc_ps_norm.ensure(size_t(tiles) * 128 * 4), "allocating locality-ordered norms");
    SSG_CK(ssg::launch_tc_norms(idx->metric == SSG_METRIC_COSINE ? SSG_METRIC_COSINE : SSG_METRIC_SQL2, x, n,
                                idx->dim, tiles * 128,
                                static_cast<float *>(idx->loc_ps_norm.p), idx->stream, &idx->last_launches, perm),
           "computing locality-ordered norms");
    SSG_CK(cudaStreamSynchronize(idx->stream), "building locality-ordered split tiles");
    idx->loc_ps_n = n;
    return SSG_OK;
}

int run_knn_tc(ssg_index *idx, const void *dq, const float *dqn, int64_t m, int k, int exclude_self,
               uint32_t *d_ids, float *d_dists, bool queries_are_db) {
    const int take = k + (exclude_self ? 1 : 0);
    const int64_t kk64 = overfetch_kk(idx, take);
    const int kp = ssg::tc_padded_k(idx->dim);
    int kk = int(kk64);
    int qt = 0, stages = 0;
    bool long_lists = false;
    idx->last_fallbacks = 0;
    // the wide scan (one query tile per CTA, two heaps per query) first when
    // it fits; longer lists on CTA pairs with one heap per query (8 KB ring
    // stages and one heap leave the list twice the room); beyond that the
    // threshold filter
    const bool wide = idx->wide_param && (ssg::tc_wide_fits(kp, kk) || (idx->pair_param && ssg::tc_pair_fits(kp, kk)));
    if (wide) qt = 1;
    else if (!ssg::tc_choose(kp, kk, &qt, &stages)) {
        if (!(idx->wide_param && idx->long_param && ssg::tc_long_fits(kp, kk)))
            return run_knn_tc_filter(idx, dq, dqn, m, k, exclude_self, d_ids, d_dists, queries_are_db, kk);
        qt = 1;
        long_lists = true;
    }
    const int64_t qrows = int64_t(qt) * 128;
    const int64_t qctas = (m + qrows - 1) / qrows;
    const int64_t n_tiles = ssg::tc_tiles(idx->n);
    int64_t splits = idx->splits_param > 0 ? idx->splits_param
                                           : wave_splits(qctas, ssg::device_sm_count(), n_tiles);
    splits = std::min<int64_t>(splits, n_tiles);
    splits = std::max<int64_t>(1, splits);
    // chunk the queries (a multiple of the CTA's query rows) to bound scratch
    const int segs = int(splits) * (long_lists ? 1 : ssg::tc_segments_per_split(qt));
    const size_t per_query = size_t(segs) * kk * 8;
    int64_t chunk = std::max<int64_t>(2 * qrows, int64_t((size_t(1) << 30) / per_query) / (2 * qrows) * (2 * qrows));
    chunk = std::min<int64_t>(chunk, (m + qrows - 1) / qrows * qrows);
    SSG_CK(idx->cand.ensure(per_query * size_t(chunk)), "allocating candidate scratch");
    SSG_CK(idx->status.ensure(sizeof(int)), "allocating the status word");
    SSG_CK(cudaMemsetAsync(idx->status.p, 0, sizeof(int), idx->stream), "clearing the status word");
    const size_t tb = ssg::tc_tile_bytes(idx->dim);
    const uint8_t *qtiles = static_cast<const uint8_t *>(idx->tc_db.p);
    const uint8_t *dtiles = static_cast<const uint8_t *>(idx->tc_db.p);
    const float *dnorm = static_cast<const float *>(idx->tc_norm.p);
    const uint32_t *perm = nullptr;
    const int *rot = nullptr;
    // allknn in one launch: scan the database in its locality order
    if (queries_are_db && idx->locality_param && !idx->capturing && m == idx->n && idx->n >= kLocalityMinRows &&
        chunk >= m && qt == 1) {
        SSG_RC(ensure_locality(idx));
        qtiles = dtiles = static_cast<const uint8_t *>(idx->loc_tiles.p);
        dnorm = static_cast<const float *>(idx->loc_norm.p);
        perm = static_cast<const uint32_t *>(idx->loc_perm.p);
        rot = static_cast<const int *>(idx->loc_rot.p);
    }
    if (!queries_are_db) {
        // an even number of tiles: the pair scan reads query tiles in pairs
        const int64_t qt_alloc = ((m + qrows - 1) / qrows * qt + 1) / 2 * 2;
        SSG_CK(idx->tc_q.ensure(size_t(qt_alloc) * tb), "allocating BF16 query tiles");
        SSG_CK(ssg::launch_bf16_tiles(static_cast<const float *>(dq), m, idx->dim, qt_alloc,
                                      static_cast<uint8_t *>(idx->tc_q.p), idx->stream, &idx->last_launches),
               "building BF16 query tiles");
        qtiles = static_cast<const uint8_t *>(idx->tc_q.p);
    }
    // every heap of a query -- its splits and the two column heaps of each
    // CTA -- shares one bound (all ones: none yet)
    uint32_t *qbound = nullptr;
    if (segs > 1) {
        SSG_CK(idx->qbound.ensure(size_t(chunk) * 4), "allocating query bounds");
        qbound = static_cast<uint32_t *>(idx->qbound.p);
    }
    for (int64_t c0 = 0; c0 < m; c0 += chunk) {
        const int64_t mc = std::min<int64_t>(chunk, m - c0);
        if (qbound) SSG_CK(cudaMemsetAsync(qbound, 0xff, size_t(mc) * 4, idx->stream), "clearing query bounds");
        if (idx->profile) SSG_CK(cudaEventRecord(idx->ev0, idx->stream), "recording an event");
        if (long_lists)
            SSG_CK(ssg::launch_tc_scan_long(idx->metric, qtiles + size_t(c0 / 128) * tb, dtiles, dnorm, idx->n, mc,
                                            idx->dim, kk, int(splits), static_cast<uint64_t *>(idx->cand.p),
                                            static_cast<int *>(idx->status.p), idx->stream, &idx->last_launches, perm,
                                            rot, idx->wave_param, qbound),
                   "launching the BF16 long-list scan kernel");
        else
            SSG_CK(ssg::launch_tc_scan(idx->metric, qtiles + size_t(c0 / 128) * tb, dtiles, dnorm, idx->n, mc,
                                       idx->dim, kk, int(splits), static_cast<uint64_t *>(idx->cand.p),
                                       static_cast<int *>(idx->status.p), idx->stream, &idx->last_launches, nullptr,
                                       perm, rot, idx->wide_param != 0, idx->wave_param, idx->pair_param != 0, qbound),
                   "launching the BF16 scan kernel");
        if (idx->profile) SSG_CK(cudaEventRecord(idx->ev1, idx->stream), "recording an event");
        ssg::FinalizeArgs f{};
        SSG_RC(reduce_segments(idx, static_cast<const uint64_t *>(idx->cand.p), mc, segs, kk, &f.cand, &f.segs));
        f.kk = kk;
        f.m = mc;
        f.k_out = k;
        f.exclude_self = exclude_self;
        f.self_base = c0;
        f.out_ids = d_ids + size_t(c0) * k;
        f.out_dists = d_dists + size_t(c0) * k;
        const size_t qrow_bytes = size_t(idx->dim) * 4;
        f.n_rows = idx->n;
        SSG_CK(ssg::launch_finalize_rerank(idx->metric, f, static_cast<const float *>(idx->db.p),
                                           static_cast<const float *>(idx->db_norm.p), idx->dim,
                                           reinterpret_cast<const float *>(static_cast<const char *>(dq) +
                                                                           size_t(c0) * qrow_bytes),
                                           dqn ? dqn + c0 : nullptr, idx->stream, &idx->last_launches),
               "launching the rerank kernel");
        if (idx->profile) {
            SSG_CK(cudaEventSynchronize(idx->ev1), "timing the scan kernel");
            float ms = 0.f;
            SSG_CK(cudaEventElapsedTime(&ms, idx->ev0, idx->ev1), "timing the scan kernel");
            idx->main_ms += ms;
            idx->main_launches += 1;
        }
    }
    if (idx->capturing) return SSG_OK;  // read after the graph launch
    int status = 0;
    SSG_CK(cudaMemcpyAsync(&status, idx->status.p, sizeof(int), cudaMemcpyDeviceToHost, idx->stream),
           "reading the status word");
    SSG_CK(cudaStreamSynchronize(idx->stream), "running the BF16 search");
    if (status != 0)
        return fail(idx, SSG_ETIMEOUT, "a bounded wait in the BF16 scan kernel gave up (code %d)", status);
    return SSG_OK;
}

// BF16 tiles of every r-th database row (the sample that sets the filter
// bounds), rebuilt when r or the database changes.
int ensure_sample_tiles(ssg_index *idx, int64_t r) {
    if (idx->smp_r == r && idx->smp_n == idx->n) return SSG_OK;
    const int64_t ns = (idx->n + r - 1) / r;
    std::vector<int64_t> rows(static_cast<size_t>(ns));
    for (int64_t i = 0; i < ns; ++i) rows[size_t(i)] = i * r;
    DevBuf list, xs;
    SSG_CK(list.ensure(size_t(ns) * 8), "allocating the sample list");
    SSG_CK(xs.ensure(size_t(ns) * idx->dim * 4), "allocating sample rows");
    SSG_CK(cudaMemcpyAsync(list.p, rows.data(), size_t(ns) * 8, cudaMemcpyHostToDevice, idx->stream),
           "copying the sample list");
    SSG_CK(ssg::launch_gather_rows(idx->db.p, static_cast<const int64_t *>(list.p), ns, size_t(idx->dim) * 4, xs.p,
                                   idx->stream, &idx->last_launches),
           "gathering sample rows");
    const int64_t tiles = (ssg::tc_tiles(ns) + 1) / 2 * 2;
    SSG_CK(idx->tc_smp.ensure(size_t(tiles) * ssg::tc_tile_bytes(idx->dim)), "allocating sample tiles");
    SSG_CK(ssg::launch_bf16_tiles(static_cast<const float *>(xs.p), ns, idx->dim, tiles,
                                  static_cast<uint8_t *>(idx->tc_smp.p), idx->stream, &idx->last_launches),
           "building sample tiles");
    SSG_CK(idx->tc_smp_norm.ensure(size_t(tiles) * 128 * 4), "allocating sample norms");
    SSG_CK(ssg::launch_tc_norms(idx->metric, static_cast<const float *>(xs.p), ns, idx->dim, tiles * 128,
                                static_cast<float *>(idx->tc_smp_norm.p), idx->stream, &idx->last_launches),
           "computing sample norms");
    SSG_CK(cudaStreamSynchronize(idx->stream), "building sample tiles");
    idx->smp_r = r;
    idx->smp_n = idx->n;
    idx->smp_rows = ns;
    return SSG_OK;
}

// The BF16 pipeline for kk beyond the on-chip heaps (e.g. long shortlists).
// A scan of every r-th database row keeps kSampleK candidates per query,
// whose distance bounds a set of about 3 * kk candidates of the full
// database; the full scan appends every candidate within the bound to the
// query's list (fcap keys), the kk best are sorted out and re-ranked exactly.
// Queries whose list came out shorter than kk or overflowed are recomputed
// with the exact direct scan.  Databases of up to 8192 rows skip the sample:
// every row is a candidate.
int run_knn_tc_filter(ssg_index *idx, const void *dq, const float *dqn, int64_t m, int k, int exclude_self,
                      uint32_t *d_ids, float *d_dists, bool queries_are_db, int kk) {
    constexpr int kSampleK = 16;
    const int64_t n = idx->n;
    const bool all = n <= 8192;
    const int fcap = all ? int(n) : 4096;
    if (kk > fcap) return fail(idx, SSG_EUNSUPPORTED, "%d candidates exceed the filter's list capacity", kk);
    const int64_t r = std::max<int64_t>(1, int64_t(3) * kk / (2 * kSampleK));
    if (!all) {
        SSG_RC(ensure_sample_tiles(idx, r));
        if (idx->smp_rows < 4 * kSampleK)
            return fail(idx, SSG_EUNSUPPORTED, "the database is too small for the filter's sample");
    }
    const int segs_s = ssg::tc_segments_per_split(1);
    const size_t per_query = size_t(fcap) * 8 + size_t(std::max(kk, segs_s * kSampleK)) * 8 + 8;
    int64_t chunk = std::max<int64_t>(256, int64_t((size_t(512) << 20) / per_query) / 256 * 256);
    chunk = std::min<int64_t>(chunk, (m + 127) / 128 * 128);
    SSG_CK(idx->f_out.ensure(size_t(chunk) * fcap * 8), "allocating filter lists");
    SSG_CK(idx->f_cnt.ensure(size_t(chunk) * 4), "allocating filter counts");
    SSG_CK(idx->f_thr.ensure(size_t(chunk) * 4), "allocating filter bounds");
    SSG_CK(idx->cand.ensure(size_t(chunk) * std::max(kk, segs_s * kSampleK) * 8), "allocating candidate scratch");
    SSG_CK(idx->flags.ensure(size_t(m) * 4 + 16), "allocating query flags");
    SSG_CK(cudaMemsetAsync(idx->flags.p, 0, size_t(m) * 4 + 16, idx->stream), "clearing query flags");
    SSG_CK(idx->status.ensure(sizeof(int)), "allocating the status word");
    SSG_CK(cudaMemsetAsync(idx->status.p, 0, sizeof(int), idx->stream), "clearing the status word");
    int *flags = static_cast<int *>(idx->flags.p);
    int *flag_count = flags + m;
    int *status = static_cast<int *>(idx->status.p);
    const size_t tb = ssg::tc_tile_bytes(idx->dim);
    const uint8_t *qtiles = static_cast<const uint8_t *>(idx->tc_db.p);
    if (!queries_are_db) {
        const int64_t qt_alloc = ((m + 127) / 128 + 1) / 2 * 2;  // even: the sample scan may run on CTA pairs
        SSG_CK(idx->tc_q.ensure(size_t(qt_alloc) * tb), "allocating BF16 query tiles");
        SSG_CK(ssg::launch_bf16_tiles(static_cast<const float *>(dq), m, idx->dim, qt_alloc,
                                      static_cast<uint8_t *>(idx->tc_q.p), idx->stream, &idx->last_launches),
               "building BF16 query tiles");
        qtiles = static_cast<const uint8_t *>(idx->tc_q.p);
    }
    const int64_t n_tiles = ssg::tc_tiles(n);
    uint64_t *cand = static_cast<uint64_t *>(idx->cand.p);
    float *thr = static_cast<float *>(idx->f_thr.p);
    int *fcnt = static_cast<int *>(idx->f_cnt.p);
    uint64_t *fout = static_cast<uint64_t *>(idx->f_out.p);
    ScanTimer timer(idx);
    for (int64_t c0 = 0; c0 < m; c0 += chunk) {
        const int64_t mc = std::min<int64_t>(chunk, m - c0);
        const int64_t qct = (mc + 127) / 128;
        const uint8_t *qc_tiles = qtiles + size_t(c0 / 128) * tb;
        if (all) {
            // 0x7f7f7f7f is a finite bound above every distance
            SSG_CK(cudaMemsetAsync(thr, 0x7f, size_t(mc) * 4, idx->stream), "setting filter bounds");
        } else {
            SSG_CK(ssg::launch_tc_scan(idx->metric, qc_tiles, static_cast<const uint8_t *>(idx->tc_smp.p),
                                       static_cast<const float *>(idx->tc_smp_norm.p), idx->smp_rows, mc, idx->dim,
                                       kSampleK, 1, cand, status, idx->stream, &idx->last_launches, nullptr,
                                       nullptr, nullptr, true, 0, idx->pair_param != 0),
                   "launching the sample scan");
            SSG_CK(ssg::launch_sample_bound(cand, mc, segs_s, kSampleK, thr, idx->stream, &idx->last_launches),
                   "computing filter bounds");
        }
        SSG_CK(cudaMemsetAsync(fcnt, 0, size_t(mc) * 4, idx->stream), "clearing filter counts");
        const int64_t splits = idx->splits_param > 0 ? std::min<int64_t>(idx->splits_param, n_tiles)
                                                     : wave_splits(qct, ssg::device_sm_count(), n_tiles);
        SSG_RC(timer.begin());
        SSG_CK(ssg::launch_tc_filter(idx->metric, qc_tiles, static_cast<const uint8_t *>(idx->tc_db.p),
                                     static_cast<const float *>(idx->tc_norm.p), n, mc, idx->dim, int(splits), thr,
                                     fout, fcnt, fcap, status, idx->stream, &idx->last_launches),
               "launching the BF16 filter scan");
        SSG_RC(timer.end());
        SSG_CK(ssg::launch_filter_select(fout, fcnt, mc, fcap, kk, cand, flags + c0, flag_count, idx->stream,
                                         &idx->last_launches),
               "selecting filtered candidates");
        ssg::FinalizeArgs f{};
        f.cand = cand;
        f.segs = 1;
        f.kk = kk;
        f.m = mc;
        f.k_out = k;
        f.exclude_self = exclude_self;
        f.self_base = c0;
        f.out_ids = d_ids + size_t(c0) * k;
        f.out_dists = d_dists + size_t(c0) * k;
        f.n_rows = idx->n;
        SSG_CK(ssg::launch_finalize_rerank(idx->metric, f, static_cast<const float *>(idx->db.p),
                                           static_cast<const float *>(idx->db_norm.p), idx->dim,
                                           static_cast<const float *>(dq) + size_t(c0) * idx->dim,
                                           dqn ? dqn + c0 : nullptr, idx->stream, &idx->last_launches),
               "launching the rerank kernel");
        SSG_RC(timer.collect());
    }
    int hstatus = 0, nflag = 0;
    SSG_CK(cudaMemcpyAsync(&hstatus, status, sizeof(int), cudaMemcpyDeviceToHost, idx->stream),
           "reading the status word");
    SSG_CK(cudaMemcpyAsync(&nflag, flag_count, sizeof(int), cudaMemcpyDeviceToHost, idx->stream), "reading flags");
    SSG_CK(cudaStreamSynchronize(idx->stream), "running the BF16 filter search");
    if (hstatus != 0)
        return fail(idx, SSG_ETIMEOUT, "a bounded wait in the BF16 scan kernel gave up (code %d)", hstatus);
    idx->last_fallbacks = nflag;
    return run_fallback(idx, static_cast<const float *>(dq), m, k, exclude_self, flags, nflag, d_ids, d_dists);
}

// The K-streaming pipeline (FP8, or BF16 for wide vectors): operand tiles
// of the queries (the database's own for allknn), the tcgen05 scan keeping
// kk = overfetch * k approximate candidates per query and split, then the
// exact FP32 rerank + (distance, id) merge.
int run_knn_stream(ssg_index *idx, const void *dq, const float *dqn, int64_t m, int k, int exclude_self,
                   uint32_t *d_ids, float *d_dists, bool queries_are_db) {
    const int fp8 = idx->prec == SSG_PREC_FP8;
    const int take = k + (exclude_self ? 1 : 0);
    const int64_t kk64 = overfetch_kk(idx, take);
    int kk = int(kk64);
    int cs = 0, stages = 0;
    const int heap_rows = ssg::stream_heap_rows(m);
    while (kk > take && !ssg::stream_choose(kk, heap_rows, &cs, &stages)) --kk;
    if (!ssg::stream_choose(kk, heap_rows, &cs, &stages))
        return fail(idx, SSG_EUNSUPPORTED, "k = %d does not fit the tensor-core kernel's on-chip top-k", take);
    const int64_t qtiles = (m + 127) / 128;
    const int64_t n_tiles = ssg::tc_tiles(idx->n);
    int64_t splits = idx->splits_param > 0 ? idx->splits_param
                                           : wave_splits(qtiles, ssg::device_sm_count(), n_tiles);
    splits = std::min<int64_t>(splits, n_tiles);
    splits = std::max<int64_t>(1, splits);
    const int segs = int(splits) * cs;
    const size_t per_query = size_t(segs) * kk * 8;
    int64_t chunk = std::max<int64_t>(128, int64_t((size_t(1) << 30) / per_query) / 128 * 128);
    chunk = std::min<int64_t>(chunk, qtiles * 128);
    SSG_CK(idx->cand.ensure(per_query * size_t(chunk)), "allocating candidate scratch");
    SSG_CK(idx->status.ensure(sizeof(int)), "allocating the status word");
    SSG_CK(cudaMemsetAsync(idx->status.p, 0, sizeof(int), idx->stream), "clearing the status word");
    const size_t tb = ssg::stream_tile_bytes(idx->dim, fp8);
    const uint8_t *qt = static_cast<const uint8_t *>(idx->st_db.p);
    const float *qgamma = fp8 ? static_cast<const float *>(idx->st_scale.p) : nullptr;
    if (!queries_are_db) {
        SSG_CK(idx->st_q.ensure(size_t(qtiles) * tb), "allocating query tiles");
        float *qs = nullptr;
        if (fp8) {
            SSG_CK(idx->st_qscale.ensure(size_t(qtiles) * 128 * 4), "allocating query scales");
            qs = static_cast<float *>(idx->st_qscale.p);
        }
        SSG_CK(ssg::launch_stream_tiles(static_cast<const float *>(dq), m, idx->dim, fp8, qtiles,
                                        static_cast<uint8_t *>(idx->st_q.p), qs, idx->stream, &idx->last_launches),
               "building query tiles");
        qt = static_cast<const uint8_t *>(idx->st_q.p);
        qgamma = qs;
    }
    // shared per-query bounds pay when many splits fill long heaps of the
    // same queries (small batches, long candidate lists): with at least kk / 2
    // heaps per query the checkpoint bounds apply (two best values per heap)
    uint32_t *gbound = nullptr;
    if (kk >= 32 && 2 * splits * cs >= kk) {
        SSG_CK(idx->gbound.ensure(size_t(chunk) * ssg::kBoundWords * 4), "allocating query bounds");
        gbound = static_cast<uint32_t *>(idx->gbound.p);
    }
    ScanTimer timer(idx);
    for (int64_t c0 = 0; c0 < m; c0 += chunk) {
        const int64_t mc = std::min<int64_t>(chunk, m - c0);
        if (gbound)
            SSG_CK(cudaMemsetAsync(gbound, 0, size_t(mc) * ssg::kBoundWords * 4, idx->stream),
                   "clearing query bounds");
        SSG_RC(timer.begin());
        SSG_CK(ssg::launch_stream_scan(qt + size_t(c0 / 128) * tb, static_cast<const uint8_t *>(idx->st_db.p),
                                       static_cast<const float *>(idx->st_alpha.p),
                                       static_cast<const float *>(idx->st_beta.p), qgamma ? qgamma + c0 : nullptr,
                                       idx->n, mc, idx->dim, fp8, kk, int(splits), heap_rows, gbound,
                                       static_cast<uint64_t *>(idx->cand.p), static_cast<int *>(idx->status.p),
                                       idx->stream, &idx->last_launches, nullptr),
               "launching the tensor-core scan kernel");
        SSG_RC(timer.end());
        ssg::FinalizeArgs f{};
        SSG_RC(reduce_segments(idx, static_cast<const uint64_t *>(idx->cand.p), mc, segs, kk, &f.cand, &f.segs));
        f.kk = kk;
        f.m = mc;
        f.k_out = k;
        f.exclude_self = exclude_self;
        f.self_base = c0;
        f.out_ids = d_ids + size_t(c0) * k;
        f.out_dists = d_dists + size_t(c0) * k;
        f.n_rows = idx->n;
        SSG_CK(ssg::launch_finalize_rerank(idx->metric, f, static_cast<const float *>(idx->db.p),
                                           static_cast<const float *>(idx->db_norm.p), idx->dim,
                                           static_cast<const float *>(dq) + size_t(c0) * idx->dim,
                                           dqn ? dqn + c0 : nullptr, idx->stream, &idx->last_launches),
               "launching the rerank kernel");
        SSG_RC(timer.collect());
    }
    if (idx->capturing) return SSG_OK;  // read after the graph launch
    int status = 0;
    SSG_CK(cudaMemcpyAsync(&status, idx->status.p, sizeof(int), cudaMemcpyDeviceToHost, idx->stream),
           "reading the status word");
    SSG_CK(cudaStreamSynchronize(idx->stream), "running the tensor-core search");
    if (status != 0)
        return fail(idx, SSG_ETIMEOUT, "a bounded wait in the tensor-core scan kernel gave up (code %d)", status);
    return SSG_OK;
}

int prepare_queries(ssg_index *idx, const void *q, int64_t m, bool src_device, const void **dq, const float **dqn) {
    const bool hamming = idx->metric == SSG_METRIC_HAMMING;
    const size_t qbytes = size_t(m) * idx->dim * (hamming ? 8 : 4);
    if (src_device && (idx->elem == SSG_ELEM_F32 || hamming)) {
        *dq = q;
    } else {
        SSG_CK(idx->qbuf.ensure(qbytes), "allocating query staging");
        int rc = upload_rows(idx, idx->qbuf.p, q, m, idx->dim, src_device);
        if (rc) return rc;
        *dq = idx->qbuf.p;
    }
    *dqn = nullptr;
    if (idx->metric == SSG_METRIC_COSINE) {
        SSG_CK(idx->qnorm.ensure(size_t(m) * 4), "allocating query norms");
        SSG_CK(ssg::launch_row_norms(static_cast<const float *>(*dq), m, idx->dim,
                                     static_cast<float *>(idx->qnorm.p), idx->stream, &idx->last_launches),
               "computing query norms");
        *dqn = static_cast<const float *>(idx->qnorm.p);
    }
    return SSG_OK;
}

int finish_call(ssg_index *idx, bool sync) {
    SSG_CK(cudaGetLastError(), "launching");
    if (sync) SSG_CK(cudaStreamSynchronize(idx->stream), "running the search");
    return SSG_OK;
}

// Serialises calls on one handle and makes its device current.  Calls that
// launch work pass `counts = true` to restart the per-call launch counter.
struct Guard {
    ssg_index *idx;
    std::unique_lock<std::mutex> lk;
    explicit Guard(ssg_index *i, bool counts = true) : idx(i), lk(i->mu) {
        cudaSetDevice(i->device);
        if (counts) i->last_launches = 0;
    }
};

double learned_recall(const ssg_index *idx) {
    bool found = false;
    return ssg::learned_get(idx->learned, "learned_recall", &found);
}

ssg::IndexView view_of(ssg_index *idx) {
    ssg::IndexView v;
    v.db = static_cast<const float *>(idx->db.p);
    v.db_norm = static_cast<const float *>(idx->db_norm.p);
    v.n = idx->n;
    v.dim = idx->dim;
    v.metric = idx->metric;
    v.stream = idx->stream;
    v.launches = &idx->last_launches;
    return v;
}

// Whether a search goes through the learned shortlist: a model exists, the
// caller has not switched it off, and its estimated recall meets the target
// (otherwise the plain exhaustive method answers: the fallback).
bool use_learned(const ssg_index *idx) {
    return idx->learned && idx->learned_param && !idx->plain_param && idx->metric != SSG_METRIC_HAMMING &&
           learned_recall(idx) >= idx->learned_target;
}

// Recall@10 of the learned pipeline against the plain method on 256 random
// objects of the database used as queries; stored with the model.
int estimate_learned_recall(ssg_index *idx, uint64_t seed) {
    const int64_t mq = std::min<int64_t>(256, idx->n);
    const int k = int(std::min<int64_t>(10, idx->n));
    std::vector<int64_t> rows(static_cast<size_t>(mq));
    uint64_t x = seed * 6364136223846793005ull + 1442695040888963407ull;
    for (auto &r : rows) {
        x = x * 6364136223846793005ull + 1442695040888963407ull;
        r = int64_t((x >> 11) % uint64_t(idx->n));
    }
    DevBuf qrows, dlist, gold, got;
    SSG_CK(dlist.ensure(size_t(mq) * 8), "allocating recall queries");
    SSG_CK(qrows.ensure(size_t(mq) * idx->dim * 4), "allocating recall queries");
    SSG_CK(gold.ensure(size_t(mq) * k * 8), "allocating recall results");
    SSG_CK(got.ensure(size_t(mq) * k * 8), "allocating recall results");
    SSG_CK(cudaMemcpyAsync(dlist.p, rows.data(), size_t(mq) * 8, cudaMemcpyHostToDevice, idx->stream), "copying");
    SSG_CK(ssg::launch_gather_rows(idx->db.p, static_cast<const int64_t *>(dlist.p), mq, size_t(idx->dim) * 4,
                                   qrows.p, idx->stream, &idx->last_launches),
           "gathering recall queries");
    const float *qn = nullptr;
    if (idx->metric == SSG_METRIC_COSINE) {
        SSG_CK(idx->qnorm.ensure(size_t(mq) * 4), "allocating query norms");
        SSG_CK(ssg::launch_row_norms(static_cast<const float *>(qrows.p), mq, idx->dim,
                                     static_cast<float *>(idx->qnorm.p), idx->stream, &idx->last_launches),
               "computing query norms");
        qn = static_cast<const float *>(idx->qnorm.p);
    }
    uint32_t *gi = static_cast<uint32_t *>(gold.p);
    float *gd = reinterpret_cast<float *>(gi + size_t(mq) * k);
    const int saved = idx->plain_param;
    idx->plain_param = 1;
    int rc = run_knn(idx, qrows.p, qn, mq, k, 0, gi, gd);
    idx->plain_param = saved;
    if (rc) return rc;
    uint32_t *li = static_cast<uint32_t *>(got.p);
    float *ld = reinterpret_cast<float *>(li + size_t(mq) * k);
    std::string err;
    rc = ssg::learned_search(idx->learned, view_of(idx), static_cast<const float *>(qrows.p), qn, mq, k, li, ld, err);
    if (rc) return fail(idx, rc, "learned search: %s", err.c_str());
    std::vector<uint32_t> hg(size_t(mq) * k), hl(size_t(mq) * k);
    SSG_CK(cudaMemcpy(hg.data(), gi, hg.size() * 4, cudaMemcpyDeviceToHost), "reading recall results");
    SSG_CK(cudaMemcpy(hl.data(), li, hl.size() * 4, cudaMemcpyDeviceToHost), "reading recall results");
    double hit = 0.0;
    for (int64_t j = 0; j < mq; ++j)
        for (int a = 0; a < k; ++a)
            for (int b = 0; b < k; ++b)
                if (hg[size_t(j) * k + a] == hl[size_t(j) * k + b]) { hit += 1.0; break; }
    ssg::learned_set_recall(idx->learned, hit / double(mq * k));
    return SSG_OK;
}

int search_locked(ssg_index *idx, const void *q, int64_t m, int32_t k, uint32_t *ids, float *dists, bool device);

// Whether a search of k neighbours on this index is a fixed sequence of
// device work with no host decisions (graph-capturable): the reduced-precision
// scans with on-chip heaps.  The plain method, the BF16 threshold filter and
// the learned path read flags on the host and run eagerly.
bool graph_capturable(ssg_index *idx, int k) {
    if (!idx->graphs_param || idx->profile || idx->plain_param || idx->prec == SSG_PREC_FP32 ||
        idx->metric == SSG_METRIC_HAMMING || use_learned(idx))
        return false;
    if (uses_stream(idx)) return true;
    int qt = 0, stages = 0;
    const int kp = ssg::tc_padded_k(idx->dim), kk = int(overfetch_kk(idx, k));
    return (idx->wide_param && (ssg::tc_wide_fits(kp, kk) || (idx->pair_param && ssg::tc_pair_fits(kp, kk)))) ||
           ssg::tc_choose(kp, kk, &qt, &stages);
}

// Everything a captured graph depends on: shape, method, tunables and the
// device buffers its nodes point at.
std::vector<uint64_t> graph_key(const ssg_index *idx, int64_t m, int k) {
    uint64_t of = 0;
    static_assert(sizeof(double) == 8, "double");
    memcpy(&of, &idx->overfetch, 8);
    std::vector<uint64_t> key = {uint64_t(m), uint64_t(k), uint64_t(idx->n), uint64_t(idx->prec),
                                 uint64_t(idx->metric), of, uint64_t(idx->splits_param), uint64_t(idx->wide_param),
                                 uint64_t(idx->wave_param), uint64_t(idx->pair_param), uint64_t(idx->long_param)};
    for (const DevBuf *b : {&idx->db, &idx->db_norm, &idx->tc_db, &idx->tc_norm, &idx->tc_q, &idx->st_db,
                            &idx->st_scale, &idx->st_alpha, &idx->st_beta, &idx->st_q, &idx->st_qscale, &idx->cand,
                            &idx->red[0], &idx->red[1], &idx->status, &idx->gbound, &idx->qnorm, &idx->pack_q,
                            &idx->pack_out, &idx->qbound})
        key.push_back(uint64_t(reinterpret_cast<uintptr_t>(b->p)));
    return key;
}

void clear_graphs(ssg_index *idx) {
    for (auto &kv : idx->graphs) cudaGraphExecDestroy(kv.second.exec);
    idx->graphs.clear();
    idx->graph_seen.clear();
}

// search_locked through the graph cache (see ssg_index::graphs), then the
// status word of the scan.
int search_graph(ssg_index *idx, const void *q, int64_t m, int32_t k, uint32_t *ids, float *dists) {
    std::vector<uint64_t> key = graph_key(idx, m, k);
    auto it = idx->graphs.find(key);
    if (it == idx->graphs.end()) {
        const bool seen = idx->graph_seen.count(key) > 0;
        if (!seen) idx->graph_seen.insert(key);
        bool captured = false;
        if (seen) {
            if (!idx->cap_stream)
                SSG_CK(cudaStreamCreateWithFlags(&idx->cap_stream, cudaStreamNonBlocking), "creating a stream");
            // the captured work must follow what is already queued on the index's stream
            SSG_CK(cudaStreamSynchronize(idx->stream), "draining the stream");
            cudaStream_t saved = idx->stream;
            const int launches0 = idx->last_launches;
            idx->stream = idx->cap_stream;
            idx->capturing = true;
            cudaError_t e = cudaStreamBeginCapture(idx->cap_stream, cudaStreamCaptureModeThreadLocal);
            int rc = e == cudaSuccess ? search_locked(idx, q, m, k, ids, dists, true) : SSG_OK;
            cudaGraph_t graph = nullptr;
            if (e == cudaSuccess) e = cudaStreamEndCapture(idx->cap_stream, &graph);
            idx->stream = saved;
            idx->capturing = false;
            cudaGraphExec_t exec = nullptr;
            if (rc == SSG_OK && e == cudaSuccess && graph) e = cudaGraphInstantiate(&exec, graph, 0);
            if (graph) cudaGraphDestroy(graph);
            if (rc == SSG_OK && e == cudaSuccess && exec && graph_key(idx, m, k) == key) {
                if (idx->graphs.size() >= 512) clear_graphs(idx);
                idx->graphs[key] = ssg_index::GraphEntry{exec, idx->last_launches - launches0};
                it = idx->graphs.find(key);
                captured = true;
            } else {
                // not capturable after all: run it eagerly (which reports
                // any genuine error of the call)
                if (exec) cudaGraphExecDestroy(exec);
                cudaGetLastError();
                idx->last_launches = launches0;
            }
        }
        if (!captured) {
            idx->last_graph = 0;
            int rc = search_locked(idx, q, m, k, ids, dists, true);
            return rc;
        }
    }
    SSG_CK(cudaGraphLaunch(it->second.exec, idx->stream), "launching a search graph");
    idx->last_launches += it->second.launches;
    idx->graph_replays += 1;
    idx->last_graph = 1;
    int status = 0;
    SSG_CK(cudaMemcpyAsync(&status, idx->status.p, sizeof(int), cudaMemcpyDeviceToHost, idx->stream),
           "reading the status word");
    SSG_CK(cudaStreamSynchronize(idx->stream), "running a search graph");
    if (status != 0)
        return fail(idx, SSG_ETIMEOUT, "a bounded wait in the tensor-core scan kernel gave up (code %d)", status);
    return SSG_OK;
}

int search_common(ssg_index *idx, const void *q, int64_t dim, int64_t m, int32_t k, uint32_t *ids,
                  float *dists, int32_t flags, bool device) {
    if (!idx) return fail(nullptr, SSG_EINVAL, "index is NULL");
    Guard g(idx);
    if (m <= 0) return fail(idx, SSG_EINVAL, "empty set of queries");
    if (dim != idx->dim)
        return fail(idx, SSG_EINVAL, "query dimension %lld does not match the index (%lld)", (long long)dim,
                    (long long)idx->dim);
    if (k <= 0) return fail(idx, SSG_EINVAL, "k must be positive (got %d)", k);
    if (!q || !ids || !dists) return fail(idx, SSG_EINVAL, "NULL query or output pointer");
    if (idx->n == 0) {
        // An empty database leaves every slot at 0 / Inf32, as searchbatch does.
        if (device) {
            return fail(idx, SSG_EINVAL, "the index is empty");
        }
        for (int64_t i = 0; i < m * int64_t(k); ++i) { ids[i] = 0; dists[i] = INFINITY; }
        return SSG_OK;
    }
    int rc = search_locked(idx, q, m, k, ids, dists, device);
    if (rc) return rc;
    return finish_call(idx, !(device && (flags & 1)));
}

// The body of a search on a locked, validated index with n > 0: query
// preparation, the learned path or the index's method, results to the host
// when !device.  Does not wait for device results.
int search_locked(ssg_index *idx, const void *q, int64_t m, int32_t k, uint32_t *ids, float *dists, bool device) {
    const void *dq;
    const float *dqn;
    int rc = prepare_queries(idx, q, m, device, &dq, &dqn);
    if (rc) return rc;
    uint32_t *d_ids = ids;
    float *d_dists = dists;
    if (!device) {
        SSG_CK(idx->outbuf.ensure(size_t(m) * k * 8), "allocating result staging");
        d_ids = static_cast<uint32_t *>(idx->outbuf.p);
        d_dists = reinterpret_cast<float *>(static_cast<char *>(idx->outbuf.p) + size_t(m) * k * 4);
    }
    idx->last_learned = 0;
    if (use_learned(idx)) {
        std::string err;
        rc = ssg::learned_search(idx->learned, view_of(idx), static_cast<const float *>(dq), dqn, m, k, d_ids, d_dists,
                                 err);
        if (rc) return fail(idx, rc, "learned search: %s", err.c_str());
        idx->last_learned = 1;
    } else {
        rc = run_knn(idx, dq, dqn, m, k, 0, d_ids, d_dists);
        if (rc) return rc;
    }
    if (!device) {
        SSG_CK(cudaMemcpyAsync(ids, d_ids, size_t(m) * k * 4, cudaMemcpyDeviceToHost, idx->stream), "copying ids");
        SSG_CK(cudaMemcpyAsync(dists, d_dists, size_t(m) * k * 4, cudaMemcpyDeviceToHost, idx->stream),
               "copying distances");
    }
    return SSG_OK;
}

int allknn_common(ssg_index *idx, int32_t k, int32_t exclude_self, uint32_t *ids, float *dists, bool device) {
    if (!idx) return fail(nullptr, SSG_EINVAL, "index is NULL");
    Guard g(idx);
    const int64_t n = idx->n;
    if (n <= 0) return fail(idx, SSG_EINVAL, "allknn needs a non-empty index");
    const int64_t kmax = exclude_self ? n - 1 : n;
    if (k <= 0 || k > kmax)
        return fail(idx, SSG_EINVAL, "allknn needs 0 < k <= %lld (got %d)", (long long)kmax, k);
    if (!ids || !dists) return fail(idx, SSG_EINVAL, "NULL output pointer");
    const float *dqn = nullptr;
    if (idx->metric == SSG_METRIC_COSINE) dqn = static_cast<const float *>(idx->db_norm.p);
    uint32_t *d_ids = ids;
    float *d_dists = dists;
    if (!device) {
        SSG_CK(idx->outbuf.ensure(size_t(n) * k * 8), "allocating result staging");
        d_ids = static_cast<uint32_t *>(idx->outbuf.p);
        d_dists = reinterpret_cast<float *>(static_cast<char *>(idx->outbuf.p) + size_t(n) * k * 4);
    }
    int rc = run_knn(idx, idx->db.p, dqn, n, k, exclude_self ? 1 : 0, d_ids, d_dists, true);
    if (rc) return rc;
    if (!device) {
        SSG_CK(cudaMemcpyAsync(ids, d_ids, size_t(n) * k * 4, cudaMemcpyDeviceToHost, idx->stream), "copying ids");
        SSG_CK(cudaMemcpyAsync(dists, d_dists, size_t(n) * k * 4, cudaMemcpyDeviceToHost, idx->stream),
               "copying distances");
    }
    return finish_call(idx, true);
}

}  // namespace

namespace ssg {
int report_error(int code, const char *msg) {
    snprintf(g_err, sizeof g_err, "%s", msg);
    return code;
}

int device_sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 148;
    if (!cached[dev]) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 148;
        cached[dev] = v;
    }
    return cached[dev];
}
}  // namespace ssg

extern "C" {

int ssg_version(void) { return 100; }

int ssg_create(int metric, int elem_type, int64_t dim, int64_t n, const void *host_db, int64_t ld,
               int precision_mode, ssg_index **out) {
    return create_common(metric, elem_type, dim, n, host_db, ld, precision_mode, out, false);
}

int ssg_create_device(int metric, int elem_type, int64_t dim, int64_t n, const void *dev_db, int64_t ld,
                      int precision_mode, ssg_index **out) {
    return create_common(metric, elem_type, dim, n, dev_db, ld, precision_mode, out, true);
}

int ssg_create_mmap(int metric, const char *path, int precision_mode, ssg_index **out) {
    if (!path || !out) return fail(nullptr, SSG_EINVAL, "NULL path or output");
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return fail(nullptr, SSG_EINVAL, "cannot open '%s'", path);
    struct stat st;
    unsigned char hdr[32];
    if (fstat(fd, &st) != 0 || st.st_size < 4096 || pread(fd, hdr, sizeof hdr, 0) != ssize_t(sizeof hdr)) {
        close(fd);
        return fail(nullptr, SSG_EINVAL, "'%s' is not a matrix database file (short header)", path);
    }
    // header (src/db/mmapmatrixdatabase.jl:10-27): magic u64 @0, version i32 @8,
    // dim i64 @12, element type code i32 @20, n i64 @24, data from byte 4096
    uint64_t magic;
    int32_t version, code;
    int64_t dim, n;
    memcpy(&magic, hdr + 0, 8);
    memcpy(&version, hdr + 8, 4);
    memcpy(&dim, hdr + 12, 8);
    memcpy(&code, hdr + 20, 4);
    memcpy(&n, hdr + 24, 8);
    int elem = -1;
    size_t es = 0;
    switch (code) {  // Float16 1, Float32 2, Float64 3, Int8 4, UInt8 5, UInt64 11
        case 1: elem = SSG_ELEM_F16; es = 2; break;
        case 2: elem = SSG_ELEM_F32; es = 4; break;
        case 3: elem = SSG_ELEM_F64; es = 8; break;
        case 4: elem = SSG_ELEM_I8; es = 1; break;
        case 5: elem = SSG_ELEM_U8; es = 1; break;
        case 11: elem = SSG_ELEM_U64; es = 8; break;
        default: break;
    }
    int rc = SSG_OK;
    if (magic != 0x4D4D444231000001ull || version != 1) {
        rc = fail(nullptr, SSG_EINVAL, "'%s' is not a matrix database file (magic / version)", path);
    } else if (elem < 0) {
        rc = fail(nullptr, SSG_EUNSUPPORTED, "element type code %d is not supported", code);
    } else if (dim <= 0 || n < 0 || (int64_t(st.st_size) - 4096) / int64_t(es) / dim < n) {
        rc = fail(nullptr, SSG_EINVAL, "corrupt matrix database file: dim %lld, n %lld, %lld bytes", (long long)dim,
                  (long long)n, (long long)st.st_size);
    }
    if (rc) {
        close(fd);
        return rc;
    }
    // map the file and upload from the mapping: pages stream from the file
    // (page cache) through the upload, no copy of the whole file in host memory
    const size_t bytes = 4096 + size_t(n) * size_t(dim) * es;
    void *map = n > 0 ? mmap(nullptr, bytes, PROT_READ, MAP_SHARED, fd, 0) : nullptr;
    close(fd);
    if (n > 0 && map == MAP_FAILED) return fail(nullptr, SSG_ENOMEM, "cannot map '%s'", path);
    if (map) madvise(map, bytes, MADV_SEQUENTIAL);
    rc = create_common(metric, elem, dim, n, map ? static_cast<const char *>(map) + 4096 : nullptr, dim,
                       precision_mode, out, false);
    if (map) munmap(map, bytes);
    return rc;
}

int ssg_search(ssg_index *idx, const void *host_q, int64_t dim, int64_t m, int32_t k, uint32_t *out_ids,
               float *out_dists, int32_t flags) {
    return search_common(idx, host_q, dim, m, k, out_ids, out_dists, flags, false);
}

int ssg_search_device(ssg_index *idx, const void *dev_q, int64_t m, int32_t k, uint32_t *dev_ids,
                      float *dev_dists, int32_t flags) {
    return search_common(idx, dev_q, idx ? idx->dim : 0, m, k, dev_ids, dev_dists, flags, true);
}

int ssg_search_batches(ssg_index *idx, int32_t nb, const void *const *dev_q, const int64_t *m, const int32_t *k,
                       uint32_t *const *dev_ids, float *const *dev_dists) {
    if (!idx) return fail(nullptr, SSG_EINVAL, "index is NULL");
    Guard g(idx);
    if (nb <= 0 || !dev_q || !m || !k || !dev_ids || !dev_dists)
        return fail(idx, SSG_EINVAL, "need nb > 0 batches and non-NULL arrays");
    int64_t mt = 0;
    // batches grouped by k: each group is one packed search with its own
    // candidate count, so a k = 1 batch never pays for a k = 100 batch's heaps
    std::map<int32_t, std::vector<int32_t>> groups;
    for (int32_t b = 0; b < nb; ++b) {
        if (m[b] < 0 || k[b] <= 0) return fail(idx, SSG_EINVAL, "batch %d: m must be >= 0 and k > 0", b);
        if (m[b] > 0 && (!dev_q[b] || !dev_ids[b] || !dev_dists[b]))
            return fail(idx, SSG_EINVAL, "batch %d: NULL query or output pointer", b);
        mt += m[b];
        if (m[b] > 0) groups[k[b]].push_back(b);
    }
    if (mt == 0) return SSG_OK;
    if (idx->n == 0) return fail(idx, SSG_EINVAL, "the index is empty");
    const size_t row_bytes = size_t(idx->dim) * elem_size(idx->elem);
    idx->last_graph = 0;
    for (const auto &grp : groups) {
        const int32_t kg = grp.first;
        int64_t mg = 0;
        for (int32_t b : grp.second) mg += m[b];
        // pack the group's queries (one copy each), one search, then each
        // batch's rows back to its own output.  Graph replays need a fixed
        // shape: the packed count is rounded up to a multiple of 32 zero rows
        // (the granularity of the small-batch heaps, so a small window keeps
        // the small-batch kernel configuration).
        const bool graph = idx->elem == SSG_ELEM_F32 && graph_capturable(idx, kg);
        const int64_t mrun = graph ? (mg + 31) / 32 * 32 : mg;
        SSG_CK(idx->pack_q.ensure(size_t(mrun) * row_bytes), "allocating packed queries");
        SSG_CK(idx->pack_out.ensure(size_t(mrun) * kg * 8), "allocating packed results");
        char *pq = static_cast<char *>(idx->pack_q.p);
        int64_t off = 0;
        for (int32_t b : grp.second) {
            SSG_CK(cudaMemcpyAsync(pq + size_t(off) * row_bytes, dev_q[b], size_t(m[b]) * row_bytes,
                                   cudaMemcpyDeviceToDevice, idx->stream),
                   "packing queries");
            off += m[b];
        }
        // padding rows repeat the group's first query: a zero query would tie
        // every database row at distance 0 under IP / NormCosine, and then its
        // heaps take every column as a candidate (slow, though still correct)
        for (int64_t done = 0; done < mrun - mg;) {
            const int64_t c = done == 0 ? 1 : std::min(done, mrun - mg - done);
            const char *src = done == 0 ? pq : pq + size_t(mg) * row_bytes;
            SSG_CK(cudaMemcpyAsync(pq + size_t(mg + done) * row_bytes, src, size_t(c) * row_bytes,
                                   cudaMemcpyDeviceToDevice, idx->stream),
                   "padding packed queries");
            done += c;
        }
        uint32_t *pi = static_cast<uint32_t *>(idx->pack_out.p);
        float *pd = reinterpret_cast<float *>(pi + size_t(mrun) * kg);
        const int rc = graph ? search_graph(idx, pq, mrun, kg, pi, pd) : search_locked(idx, pq, mg, kg, pi, pd, true);
        if (rc) return rc;
        off = 0;
        for (int32_t b : grp.second) {
            SSG_CK(cudaMemcpyAsync(dev_ids[b], pi + size_t(off) * kg, size_t(m[b]) * kg * 4,
                                   cudaMemcpyDeviceToDevice, idx->stream),
                   "unpacking ids");
            SSG_CK(cudaMemcpyAsync(dev_dists[b], pd + size_t(off) * kg, size_t(m[b]) * kg * 4,
                                   cudaMemcpyDeviceToDevice, idx->stream),
                   "unpacking distances");
            off += m[b];
        }
    }
    return finish_call(idx, true);
}

int ssg_allknn(ssg_index *idx, int32_t k, int32_t exclude_self, uint32_t *out_ids, float *out_dists) {
    return allknn_common(idx, k, exclude_self, out_ids, out_dists, false);
}

int ssg_allknn_device(ssg_index *idx, int32_t k, int32_t exclude_self, uint32_t *dev_ids, float *dev_dists) {
    return allknn_common(idx, k, exclude_self, dev_ids, dev_dists, true);
}

int ssg_append(ssg_index *idx, const void *host_rows, int64_t count) {
    if (!idx) return fail(nullptr, SSG_EINVAL, "index is NULL");
    Guard g(idx);
    if (count < 0) return fail(idx, SSG_EINVAL, "negative count");
    if (count == 0) return SSG_OK;
    if (!host_rows) return fail(idx, SSG_EINVAL, "rows pointer is NULL");
    if (idx->n + count >= (int64_t(1) << 32) - 1) return fail(idx, SSG_EINVAL, "too many objects");
    int rc = add_rows(idx, host_rows, count, idx->dim, false);
    if (rc || !idx->learned) return rc;
    // the learned shortlist must cover the new objects: embed the database again
    std::string err;
    rc = ssg::learned_index_db(idx->learned, view_of(idx), err);
    if (rc) return fail(idx, rc, "re-indexing the learned shortlist: %s", err.c_str());
    return SSG_OK;
}

int ssg_rerank(ssg_index *idx, const void *host_q, int64_t m, int32_t len, uint32_t *ids, float *dists) {
    if (!idx) return fail(nullptr, SSG_EINVAL, "index is NULL");
    Guard g(idx);
    if (m <= 0) return fail(idx, SSG_EINVAL, "empty set of queries");
    if (len <= 0) return fail(idx, SSG_EINVAL, "candidate lists must be non-empty");
    if (len > 16384) return fail(idx, SSG_EUNSUPPORTED, "candidate lists longer than 16384 are not supported");
    if (!host_q || !ids || !dists) return fail(idx, SSG_EINVAL, "NULL pointer");
    for (int64_t i = 0; i < m * int64_t(len); ++i)
        if (ids[i] > idx->n) return fail(idx, SSG_EINVAL, "candidate id %u out of range 1..%lld", ids[i], (long long)idx->n);
    const void *dq;
    const float *dqn;
    int rc = prepare_queries(idx, host_q, m, false, &dq, &dqn);
    if (rc) return rc;
    SSG_CK(idx->outbuf.ensure(size_t(m) * len * 8), "allocating rerank staging");
    uint32_t *d_ids = static_cast<uint32_t *>(idx->outbuf.p);
    float *d_d = reinterpret_cast<float *>(static_cast<char *>(idx->outbuf.p) + size_t(m) * len * 4);
    SSG_CK(cudaMemcpyAsync(d_ids, ids, size_t(m) * len * 4, cudaMemcpyHostToDevice, idx->stream), "copying ids");
    SSG_CK(cudaMemcpyAsync(d_d, dists, size_t(m) * len * 4, cudaMemcpyHostToDevice, idx->stream), "copying dists");
    SSG_CK(ssg::launch_rerank(idx->metric, idx->db.p, static_cast<const float *>(idx->db_norm.p), idx->dim, dq, dqn,
                              m, len, d_ids, d_d, idx->stream, &idx->last_launches),
           "launching rerank");
    SSG_CK(cudaMemcpyAsync(ids, d_ids, size_t(m) * len * 4, cudaMemcpyDeviceToHost, idx->stream), "copying ids");
    SSG_CK(cudaMemcpyAsync(dists, d_d, size_t(m) * len * 4, cudaMemcpyDeviceToHost, idx->stream), "copying dists");
    return finish_call(idx, true);
}

int ssg_set_param(ssg_index *idx, const char *key, double value) {
    if (!idx || !key) return fail(idx, SSG_EINVAL, "NULL index or key");
    Guard g(idx, false);
    std::string k(key);
    if (k == "splits") {
        if (value < 0 || value > 65535) return fail(idx, SSG_EINVAL, "splits out of range");
        idx->splits_param = int(value);
    } else if (k == "overfetch") {
        if (!(value >= 1.0 && value <= 64.0)) return fail(idx, SSG_EINVAL, "overfetch must be in [1, 64]");
        idx->overfetch = value;
    } else if (k == "margin") {
        if (value < 0 || value > 4096) return fail(idx, SSG_EINVAL, "margin out of range");
        idx->margin_param = int(value);
    } else if (k == "exact_scan") {
        idx->exact_scan_param = value != 0.0;
    } else if (k == "plain") {
        idx->plain_param = value != 0.0;
    } else if (k == "plain_tc") {
        idx->plain_tc_param = value != 0.0;
    } else if (k == "learned") {
        idx->learned_param = value != 0.0;
    } else if (k == "learned_target") {
        if (!(value >= 0.0 && value <= 1.0)) return fail(idx, SSG_EINVAL, "learned_target must be in [0, 1]");
        idx->learned_target = value;
    } else if (k == "train_hard") {
        if (!(value >= 0.0 && value <= 1.0)) return fail(idx, SSG_EINVAL, "train_hard must be in [0, 1]");
        idx->train_hard = value;
    } else if (k == "shortlist") {
        if (!(value >= 1 && value <= 4096)) return fail(idx, SSG_EINVAL, "shortlist must be in [1, 4096]");
        if (!ssg::learned_set(idx->learned, "shortlist", value))
            return fail(idx, SSG_EINVAL, "no learned model on this index");
        // the recall estimate belongs to the shortlist length: measure it again
        return estimate_learned_recall(idx, 12345);
    } else if (k == "graphs") {
        idx->graphs_param = value != 0.0;
        if (!idx->graphs_param) clear_graphs(idx);
    } else if (k == "locality") {
        idx->locality_param = value != 0.0;
    } else if (k == "wide") {
        idx->wide_param = value != 0.0;
    } else if (k == "pair") {
        idx->pair_param = value != 0.0;
    } else if (k == "long_lists") {
        idx->long_param = value != 0.0;
    } else if (k == "locality_rows" || k == "locality_chain") {
        if (k == "locality_rows") {
            if (!(value >= 64 && value <= 65536)) return fail(idx, SSG_EINVAL, "locality_rows out of range");
            idx->loc_rows_param = int64_t(value);
        } else {
            idx->loc_chain_param = value != 0.0;
        }
        idx->loc_n = idx->loc_bf16_n = idx->loc_ps_n = -1;  // rebuilt on the next allknn
    } else if (k == "wave") {
        if (!(value >= 0 && value <= 1e6)) return fail(idx, SSG_EINVAL, "wave out of range");
        idx->wave_param = int64_t(value);
    } else if (k == "profile") {
        idx->profile = value != 0.0;
        if (idx->profile) { idx->main_ms = 0.0; idx->main_launches = 0; }
    } else {
        return fail(idx, SSG_EINVAL, "unknown parameter '%s'", key);
    }
    return SSG_OK;
}

int ssg_get_param(ssg_index *idx, const char *key, double *value) {
    if (!idx || !key || !value) return fail(idx, SSG_EINVAL, "NULL argument");
    Guard g(idx, false);
    std::string k(key);
    if (k == "n") *value = double(idx->n);
    else if (k == "dim") *value = double(idx->dim);
    else if (k == "metric") *value = idx->metric;
    else if (k == "precision") *value = idx->prec;
    else if (k == "splits") *value = idx->splits_param;
    else if (k == "overfetch") *value = idx->overfetch;
    else if (k == "profile") *value = idx->profile;
    else if (k == "locality") *value = idx->locality_param;
    else if (k == "wide") *value = idx->wide_param;
    else if (k == "wave") *value = double(idx->wave_param);
    else if (k == "pair") *value = idx->pair_param;
    else if (k == "graphs") *value = idx->graphs_param;
    else if (k == "graph_replays") *value = double(idx->graph_replays);
    else if (k == "last_graph") *value = idx->last_graph;
    else if (k == "main_kernel_ms") *value = idx->main_ms;
    else if (k == "main_kernel_launches") *value = double(idx->main_launches);
    else if (k == "kernel_launches") *value = idx->last_launches;
    else if (k == "margin") *value = idx->margin_param;
    else if (k == "exact_scan") *value = idx->exact_scan_param;
    else if (k == "plain") *value = idx->plain_param;
    else if (k == "plain_tc") *value = idx->plain_tc_param;
    else if (k == "long_lists") *value = idx->long_param;
    else if (k == "locality_rows") *value = double(idx->loc_rows_param);
    else if (k == "locality_chain") *value = idx->loc_chain_param;
    else if (k == "last_plain_tc") *value = idx->last_plain_tc;
    else if (k == "learned") *value = idx->learned_param;
    else if (k == "learned_target") *value = idx->learned_target;
    else if (k == "train_hard") *value = idx->train_hard;
    else if (k == "learned_used") *value = idx->last_learned;
    else if (k == "fallbacks") *value = idx->last_fallbacks;
    else if (k == "max_x_sq") *value = idx->max_x_sq;
    else if (k == "device_bytes")
        *value = double(idx->db.bytes + idx->db_norm.bytes + idx->qbuf.bytes + idx->qnorm.bytes + idx->cand.bytes +
                        idx->gheap.bytes + idx->outbuf.bytes + idx->stage.bytes + idx->tc_db.bytes +
                        idx->tc_norm.bytes + idx->tc_q.bytes);
    else {
        bool found = false;
        const double v = ssg::learned_get(idx->learned, key, &found);
        if (!found) return fail(idx, SSG_EINVAL, "unknown parameter '%s'", key);
        *value = v;
    }
    return SSG_OK;
}

int ssg_set_stream(ssg_index *idx, void *stream) {
    if (!idx) return fail(nullptr, SSG_EINVAL, "index is NULL");
    Guard g(idx);
    if (idx->own_stream && idx->stream) cudaStreamDestroy(idx->stream);
    idx->stream = static_cast<cudaStream_t>(stream);
    idx->own_stream = false;
    return SSG_OK;
}

int ssg_last_error(ssg_index *idx, char *buf, int64_t len) {
    const char *src = idx ? idx->err : g_err;
    int full = int(strlen(src));
    if (buf && len > 0) {
        int64_t c = std::min<int64_t>(full, len - 1);
        memcpy(buf, src, size_t(c));
        buf[c] = '\0';
    }
    return full;
}

int ssg_closestpairs(ssg_index *idx, const void *host_B, int64_t m, int32_t k, int32_t min_k, int32_t samedata,
                     int32_t *out_i, int32_t *out_j, float *out_d, int64_t *count) {
    if (!idx) return fail(nullptr, SSG_EINVAL, "index is NULL");
    Guard g(idx);
    if (k <= 0 || min_k < k || min_k > 4096)
        return fail(idx, SSG_EINVAL, "closest pairs need 0 < k <= min_k <= 4096 (got k = %d, min_k = %d)", k, min_k);
    if (!out_i || !out_j || !out_d || !count) return fail(idx, SSG_EINVAL, "NULL output pointer");
    const bool own = host_B == nullptr;  // B is the indexed database itself
    if (own) {
        m = idx->n;
        samedata = 1;
    }
    if (m < 0) return fail(idx, SSG_EINVAL, "negative number of objects");
    for (int32_t r = 0; r < k; ++r) { out_i[r] = 0; out_j[r] = 0; out_d[r] = INFINITY; }
    *count = 0;
    const int64_t avail = idx->n - (samedata ? 1 : 0);
    if (m == 0 || avail <= 0) return SSG_OK;
    const int kk = int(std::min<int64_t>(min_k, avail));
    // 1. each object of B: its kk nearest objects of the index (itself excluded)
    const void *dq;
    const float *dqn = nullptr;
    if (own) {
        dq = idx->db.p;
        if (idx->metric == SSG_METRIC_COSINE) dqn = static_cast<const float *>(idx->db_norm.p);
    } else {
        int rc = prepare_queries(idx, host_B, m, false, &dq, &dqn);
        if (rc) return rc;
    }
    if (int64_t(m) * kk >= (int64_t(1) << 32) - 1) return fail(idx, SSG_EUNSUPPORTED, "too many candidate pairs");
    SSG_CK(idx->pack_out.ensure(size_t(m) * kk * 8), "allocating pair candidates");
    uint32_t *ids = static_cast<uint32_t *>(idx->pack_out.p);
    float *dists = reinterpret_cast<float *>(ids + size_t(m) * kk);
    int rc = run_knn(idx, dq, dqn, m, kk, samedata ? 1 : 0, ids, dists, own);
    if (rc) return rc;
    // 2. the k smallest of the m sorted rows, merged as segments of one list
    SSG_CK(idx->pack_q.ensure(size_t(m) * kk * 8), "allocating pair keys");
    uint64_t *keys = static_cast<uint64_t *>(idx->pack_q.p);
    SSG_CK(ssg::launch_pair_keys(ids, dists, int64_t(m) * kk, keys, idx->stream, &idx->last_launches),
           "building pair keys");
    ssg::FinalizeArgs f{};
    SSG_RC(reduce_segments(idx, keys, 1, int(std::min<int64_t>(m, INT32_MAX)), kk, &f.cand, &f.segs));
    DevBuf sel;
    SSG_CK(sel.ensure(size_t(k) * 8 + size_t(k) * 12), "allocating the selection");
    uint32_t *sel_ids = static_cast<uint32_t *>(sel.p);
    float *sel_d = reinterpret_cast<float *>(sel_ids + k);
    f.kk = kk;
    f.m = 1;
    f.k_out = k;
    f.exclude_self = 0;
    f.self_base = 0;
    f.out_ids = sel_ids;
    f.out_dists = sel_d;
    SSG_CK(ssg::launch_finalize(f, idx->stream, &idx->last_launches), "merging pair candidates");
    int32_t *di = reinterpret_cast<int32_t *>(sel_d + k);
    int32_t *dj = di + k;
    float *dd = reinterpret_cast<float *>(dj + k);
    SSG_CK(ssg::launch_pair_decode(sel_ids, sel_d, k, ids, kk, di, dj, dd, idx->stream, &idx->last_launches),
           "decoding pairs");
    SSG_CK(cudaMemcpyAsync(out_i, di, size_t(k) * 4, cudaMemcpyDeviceToHost, idx->stream), "copying pairs");
    SSG_CK(cudaMemcpyAsync(out_j, dj, size_t(k) * 4, cudaMemcpyDeviceToHost, idx->stream), "copying pairs");
    SSG_CK(cudaMemcpyAsync(out_d, dd, size_t(k) * 4, cudaMemcpyDeviceToHost, idx->stream), "copying pairs");
    SSG_CK(cudaStreamSynchronize(idx->stream), "finding closest pairs");
    int64_t c = 0;
    while (c < k && out_i[c] != 0) ++c;
    *count = c;
    return SSG_OK;
}

int ssg_bitsketch(const void *dev_R, int64_t dim, int64_t outdim, const void *dev_X, int64_t n, uint64_t *dev_out,
                  void *stream) {
    if (dim <= 0 || outdim <= 0 || n < 0 || outdim > (int64_t(1) << 24) || dim > (int64_t(1) << 24))
        return fail(nullptr, SSG_EINVAL, "bitsketch needs dim > 0 and 0 < outdim <= 2^24");
    if (n == 0) return SSG_OK;
    if (!dev_R || !dev_X || !dev_out) return fail(nullptr, SSG_EINVAL, "NULL buffer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t tf = ssg::gemm_tile_floats(dim);
    const int64_t xt = (n + 127) / 128, rt = (outdim + 127) / 128;
    void *xtiles = nullptr, *rtiles = nullptr;
    cudaError_t e = cudaMallocAsync(&xtiles, size_t(xt) * tf * 4, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&rtiles, size_t(rt) * tf * 4, st);
    int launches = 0;
    if (e == cudaSuccess)
        e = ssg::launch_gemm_tiles(static_cast<const float *>(dev_X), n, dim, xt, static_cast<float *>(xtiles), st,
                                   &launches);
    if (e == cudaSuccess)
        e = ssg::launch_gemm_tiles(static_cast<const float *>(dev_R), outdim, dim, rt, static_cast<float *>(rtiles),
                                   st, &launches);
    if (e == cudaSuccess)
        e = ssg::launch_bitsketch(static_cast<const float *>(xtiles), static_cast<const float *>(rtiles), dim, n,
                                  outdim, dev_out, st, &launches);
    if (xtiles) cudaFreeAsync(xtiles, st);
    if (rtiles) cudaFreeAsync(rtiles, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(nullptr, e == cudaErrorMemoryAllocation ? SSG_ENOMEM : SSG_ECUDA, "bitsketch: %s",
                    cudaGetErrorString(e));
    }
    return SSG_OK;
}

int ssg_train_mlp(ssg_index *idx, int64_t sample_n, int64_t triplets, int32_t epochs, int32_t hidden,
                  int32_t out_dim, int32_t batch, double lr, uint64_t seed) {
    if (!idx) return fail(nullptr, SSG_EINVAL, "index is NULL");
    Guard g(idx);
    if (idx->metric == SSG_METRIC_HAMMING)
        return fail(idx, SSG_EUNSUPPORTED, "the learned shortlist is for float metrics");
    if (idx->n < 32) return fail(idx, SSG_EINVAL, "the index needs at least 32 objects to train on");
    if (sample_n < 12 || triplets < 0 || epochs < 0 || hidden < 0 || hidden > 8192 || out_dim < 1 ||
        out_dim > 256 || batch < 1 || batch > 65536 || !(lr > 0.0))
        return fail(idx, SSG_EINVAL, "invalid training arguments");
    ssg::TrainArgs t{};
    t.sample = sample_n;
    t.triplets = triplets;
    t.epochs = epochs;
    t.hidden = hidden;
    t.out_dim = out_dim;
    t.batch = batch;
    t.lr = float(lr);
    t.margin = 1.0f;
    t.seed = seed;
    t.shortlist = 512;
    t.hard = float(idx->train_hard);
    ssg::LearnedModel *m = nullptr;
    std::string err;
    int rc = ssg::learned_train(view_of(idx), t, &m, err);
    if (rc) return fail(idx, rc, "training failed: %s", err.c_str());
    ssg::learned_free(idx->learned);
    idx->learned = m;
    return estimate_learned_recall(idx, seed);
}

int ssg_save_model(ssg_index *idx, const char *path) {
    if (!idx || !path) return fail(idx, SSG_EINVAL, "NULL argument");
    Guard g(idx, false);
    if (!idx->learned) return fail(idx, SSG_EINVAL, "no learned model on this index");
    std::string err;
    int rc = ssg::learned_save(idx->learned, path, err);
    return rc ? fail(idx, rc, "%s", err.c_str()) : SSG_OK;
}

int ssg_load_model(ssg_index *idx, const char *path) {
    if (!idx || !path) return fail(idx, SSG_EINVAL, "NULL argument");
    Guard g(idx);
    ssg::LearnedModel *m = nullptr;
    std::string err;
    int rc = ssg::learned_load(view_of(idx), path, &m, err);
    if (rc) return fail(idx, rc, "%s", err.c_str());
    ssg::learned_free(idx->learned);
    idx->learned = m;
    return estimate_learned_recall(idx, 12345);
}

int ssg_mlp_grad_check(int64_t d, int64_t hidden, int64_t out_dim, const float *W1, const float *b1, const float *W2,
                       const float *b2, const float *X, int32_t batch, float margin, float *loss, float *gW1,
                       float *gb1, float *gW2, float *gb2) {
    if (d <= 0 || hidden <= 0 || out_dim <= 0 || batch <= 0 || !W1 || !b1 || !W2 || !b2 || !X || !loss || !gW1 ||
        !gb1 || !gW2 || !gb2)
        return fail(nullptr, SSG_EINVAL, "invalid gradient-check arguments");
    std::string err;
    int rc = ssg::learned_grad_check(d, hidden, out_dim, W1, b1, W2, b2, X, batch, margin, loss, gW1, gb1, gW2, gb2,
                                     err);
    return rc ? fail(nullptr, rc, "%s", err.c_str()) : SSG_OK;
}

void ssg_destroy(ssg_index *idx) {
    if (!idx) return;
    cudaSetDevice(idx->device);
    if (idx->stream) cudaStreamSynchronize(idx->stream);
    idx->db.release();
    idx->db_norm.release();
    idx->qbuf.release();
    idx->qnorm.release();
    idx->qraw.release();
    idx->cand.release();
    idx->gheap.release();
    idx->outbuf.release();
    idx->stage.release();
    idx->tc_db.release();
    idx->tc_norm.release();
    idx->tc_q.release();
    idx->status.release();
    for (DevBuf *b : {&idx->loc_perm, &idx->loc_rot, &idx->loc_tiles, &idx->loc_norm, &idx->loc_ps_db,
                      &idx->loc_ps_dbq, &idx->loc_ps_norm})
        b->release();
    ssg::learned_free(idx->learned);
    idx->learned = nullptr;
    for (DevBuf *b : {&idx->st_db, &idx->st_scale, &idx->st_alpha, &idx->st_beta, &idx->st_q, &idx->st_qscale,
                      &idx->red[0], &idx->red[1]})
        b->release();
    for (DevBuf *b : {&idx->sq_norm, &idx->sq_max, &idx->flags, &idx->qsq, &idx->fb_list, &idx->fb_q, &idx->fb_out,
                      &idx->fb_cand, &idx->fb_qn, &idx->tc_smp, &idx->tc_smp_norm, &idx->f_out, &idx->f_cnt,
                      &idx->f_thr, &idx->gbound, &idx->pack_q, &idx->pack_out, &idx->gm_db, &idx->gm_q,
                      &idx->ps_db, &idx->ps_dbq, &idx->ps_norm, &idx->ps_q, &idx->qbound, &idx->pss_db,
                      &idx->pss_dbq, &idx->pss_alpha, &idx->pss_beta, &idx->pss_q})
        b->release();
    if (idx->ev0) cudaEventDestroy(idx->ev0);
    if (idx->ev1) cudaEventDestroy(idx->ev1);
    clear_graphs(idx);
    if (idx->cap_stream) cudaStreamDestroy(idx->cap_stream);
    if (idx->own_stream && idx->stream) cudaStreamDestroy(idx->stream);
    delete idx;
}

}  // extern "C"
