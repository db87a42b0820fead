/*
 * knn_oracle.c -- CPU restatement of SimilaritySearch.jl's exhaustive k-NN path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GPU engine is
 * checked against.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline / reference arm load it; the product library never links it and
 * never falls back to it.
 *
 * Every function restates the reference algorithm (SimilaritySearch.jl 1.2.0)
 * and cites the Julia source it follows:
 *   - KnnSorted push / insert-after-equal / reject >= frontier:
 *       src/pqueue/knnsorted.jl:68-101, 140-168
 *   - ExhaustiveSearch.search (loop order, evaluate(dist, db[i], q), 1-based ids):
 *       src/exact/sequential-exhaustive.jl:68-80
 *   - ParallelExhaustiveSearch.search (contiguous chunks, per-chunk KnnSorted,
 *     merge in batch order):  src/exact/parallel-exhaustive.jl:64-102,
 *       src/parallel.jl:606-614 (Iterators.partition), src/SimilaritySearch.jl:101-111
 *   - searchbatch! (output init 0 / Inf32, column j = query j):
 *       src/SimilaritySearch.jl:309-348
 *   - allknn! (self kept in the result):  src/allknn.jl:66-110
 *   - distances:  src/dist/vecs.jl:59-67 (L2), 93-102 (SqL2);
 *       src/dist/cos.jl:76-84 (NormCosine, Float32 method), 103 (Cosine);
 *       src/dist/bits.jl:18-25 (Hamming);  src/dist/vecs-cast-f32.jl:76-93,148-189
 *   - rerank!:  src/rerank.jl:22-41
 *   - recallscore / macrorecall:  src/perf.jl:31-33, 71-79
 *
 * Summation order.  The reference sums with `@fastmath @simd muladd`, which lets
 * LLVM reassociate into host-SIMD-width partial sums.  The oracle takes a
 * `lanes` argument: lanes == 1 sums sequentially with fmaf (the order the GPU
 * kernels use, so the two agree bit for bit); lanes == L keeps L partial sums
 * (element i goes to lane i mod L), combines them as a pairwise tree and adds
 * the scalar remainder, the shape of an LLVM-vectorised loop.  Both are valid
 * executions of the reference's reassociable loop.
 *
 * Inner product (`metric 4`) has no reference type: it is -dot(x, q), i.e.
 * NormCosine minus one, ranking by maximum inner product.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum {
    M_SQL2 = 0, M_L2 = 1, M_NORMCOSINE = 2, M_COSINE = 3, M_IP = 4, M_HAMMING = 5
};

/* ------------------------------------------------------------------ */
/* KnnSorted (src/pqueue/knnsorted.jl).  sp/ep are 1-based like Julia. */
/* ------------------------------------------------------------------ */

/* sort_last_item! (knnsorted.jl:68-101): binary search for the first
 * position whose dist is > item (so an equal item goes AFTER existing equal
 * ones), then block shift. Arrays are indexed 1-based through the -1 offset. */
static void sort_last_item(uint32_t *ids, float *dists, int32_t sp, int32_t ep)
{
    if (sp == ep) return;
    uint32_t item_id = ids[ep - 1];
    float item_dist = dists[ep - 1];
    if (dists[ep - 2] <= item_dist) return;
    int32_t lo = sp, hi = ep - 1;
    while (lo < hi) {
        int32_t mid = (int32_t)(((uint32_t)lo + (uint32_t)hi) >> 1);
        if (dists[mid - 1] <= item_dist) lo = mid + 1;
        else hi = mid;
    }
    for (int32_t i = ep; i >= lo + 1; --i) ids[i - 1] = ids[i - 2];
    ids[lo - 1] = item_id;
    for (int32_t i = ep; i >= lo + 1; --i) dists[i - 1] = dists[i - 2];
    dists[lo - 1] = item_dist;
}

/* push_item!(::KnnSorted, ::IdDist) (knnsorted.jl:140-168).
 * cap = length(ids) (backing storage), maxlen = k.  Returns 1 if inserted. */
int oracle_knnsorted_push(uint32_t *ids, float *dists, int32_t cap,
                          int32_t *sp_, int32_t *ep_, int32_t maxlen,
                          uint32_t id, float d)
{
    int32_t sp = *sp_, ep = *ep_;
    int32_t len = ep - sp + 1;
    if (len < maxlen) {
        if (ep == cap) { /* reorganise: shift the active range to the front */
            int32_t n = ep - sp + 1;
            for (int32_t i = 1; i <= n; ++i) {
                ids[i - 1] = ids[sp + i - 2];
                dists[i - 1] = dists[sp + i - 2];
            }
            sp = 1; ep = n;
        }
        ep += 1;
        ids[ep - 1] = id;
        dists[ep - 1] = d;
        sort_last_item(ids, dists, sp, ep);
        *sp_ = sp; *ep_ = ep;
        return 1;
    }
    /* `item.dist >= maximum(res) && return false` (knnsorted.jl:163) */
    if (d >= dists[ep - 1]) return 0;
    ids[ep - 1] = id;
    dists[ep - 1] = d;
    sort_last_item(ids, dists, sp, ep);
    return 1;
}

/* ------------------------------------------------------------------ */
/* Distances                                                           */
/* ------------------------------------------------------------------ */

/* Tree-combine L partial sums the way a vector reduction does: halve. */
static float tree_reduce(float *p, int L)
{
    while (L > 1) {
        int h = L / 2;
        for (int i = 0; i < h; ++i) p[i] = p[i] + p[i + h];
        if (L & 1) p[0] = p[0] + p[L - 1];
        L = h;
    }
    return p[0];
}

#define MAXLANES 64

/* sum_i (a_i - b_i)^2 with muladd (vecs.jl:93-102). */
static float sq_l2(const float *a, const float *b, int64_t dim, int lanes)
{
    if (lanes <= 1) {
        float d = 0.0f;
        for (int64_t i = 0; i < dim; ++i) {
            float m = a[i] - b[i];
            d = fmaf(m, m, d);
        }
        return d;
    }
    float p[MAXLANES];
    if (lanes > MAXLANES) lanes = MAXLANES;
    for (int l = 0; l < lanes; ++l) p[l] = 0.0f;
    int64_t body = (dim / lanes) * lanes;
    for (int64_t i = 0; i < body; i += lanes)
        for (int l = 0; l < lanes; ++l) {
            float m = a[i + l] - b[i + l];
            p[l] = fmaf(m, m, p[l]);
        }
    float d = tree_reduce(p, lanes);
    for (int64_t i = body; i < dim; ++i) {
        float m = a[i] - b[i];
        d = fmaf(m, m, d);
    }
    return d;
}

/* sum_i a_i * b_i with muladd (cos.jl:78-84, vecs-cast-f32.jl:76-84). */
static float dot32(const float *a, const float *b, int64_t dim, int lanes)
{
    if (lanes <= 1) {
        float d = 0.0f;
        for (int64_t i = 0; i < dim; ++i) d = fmaf(a[i], b[i], d);
        return d;
    }
    float p[MAXLANES];
    if (lanes > MAXLANES) lanes = MAXLANES;
    for (int l = 0; l < lanes; ++l) p[l] = 0.0f;
    int64_t body = (dim / lanes) * lanes;
    for (int64_t i = 0; i < body; i += lanes)
        for (int l = 0; l < lanes; ++l) p[l] = fmaf(a[i + l], b[i + l], p[l]);
    float d = tree_reduce(p, lanes);
    for (int64_t i = body; i < dim; ++i) d = fmaf(a[i], b[i], d);
    return d;
}

static float hamming(const uint64_t *a, const uint64_t *b, int64_t words)
{
    int64_t d = 0;
    for (int64_t i = 0; i < words; ++i) d += __builtin_popcountll(a[i] ^ b[i]);
    return (float)d;
}

/* evaluate(dist, a, b) with a = db[i], b = q (sequential-exhaustive.jl:74). */
float oracle_evaluate(int metric, const void *a_, const void *b_, int64_t dim, int lanes)
{
    if (metric == M_HAMMING)
        return hamming((const uint64_t *)a_, (const uint64_t *)b_, dim);
    const float *a = (const float *)a_, *b = (const float *)b_;
    switch (metric) {
    case M_SQL2: return sq_l2(a, b, dim, lanes);
    case M_L2: return sqrtf(sq_l2(a, b, dim, lanes));
    case M_NORMCOSINE: return 1.0f - dot32(a, b, dim, lanes);
    case M_IP: return -dot32(a, b, dim, lanes);
    case M_COSINE: {
        /* one - dot(a,b) / (norm(a) * norm(b))  (cos.jl:103) */
        float d = dot32(a, b, dim, lanes);
        float na = sqrtf(dot32(a, a, dim, lanes));
        float nb = sqrtf(dot32(b, b, dim, lanes));
        return 1.0f - d / (na * nb);
    }
    default: return NAN;
    }
}

/* FP64 evaluation of the same formulas (used for recall / max|dd| checks). */
double oracle_evaluate_f64(int metric, const void *a_, const void *b_, int64_t dim)
{
    if (metric == M_HAMMING)
        return (double)hamming((const uint64_t *)a_, (const uint64_t *)b_, dim);
    const float *a = (const float *)a_, *b = (const float *)b_;
    double s = 0.0, na = 0.0, nb = 0.0;
    switch (metric) {
    case M_SQL2:
    case M_L2:
        for (int64_t i = 0; i < dim; ++i) { double m = (double)a[i] - (double)b[i]; s += m * m; }
        return metric == M_L2 ? sqrt(s) : s;
    case M_NORMCOSINE:
    case M_IP:
        for (int64_t i = 0; i < dim; ++i) s += (double)a[i] * (double)b[i];
        return metric == M_IP ? -s : 1.0 - s;
    case M_COSINE:
        for (int64_t i = 0; i < dim; ++i) {
            s += (double)a[i] * (double)b[i];
            na += (double)a[i] * (double)a[i];
            nb += (double)b[i] * (double)b[i];
        }
        return 1.0 - s / (sqrt(na) * sqrt(nb));
    default: return NAN;
    }
}

static inline const void *row_ptr(int metric, const void *base, int64_t dim, int64_t i)
{
    if (metric == M_HAMMING) return (const uint64_t *)base + i * dim;
    return (const float *)base + i * dim;
}

/* ------------------------------------------------------------------ */
/* search(::ExhaustiveSearch, ctx, q, res)  (sequential-exhaustive.jl:68-80)  */
/* ------------------------------------------------------------------ */

/* Fills one output column (k slots) the way knnqueue(ctx, view(ids,:,j),
 * view(dists,:,j)) + search do: the queue starts empty over the column, so
 * slots that are never reached keep their initial 0 / Inf32. */
void oracle_search(int metric, const void *db, int64_t dim, int64_t n,
                   const void *q, int32_t k, uint32_t *ids, float *dists, int lanes)
{
    int32_t sp = 1, ep = 0;
    for (int64_t i = 1; i <= n; ++i) {
        float d = oracle_evaluate(metric, row_ptr(metric, db, dim, i - 1), q, dim, lanes);
        oracle_knnsorted_push(ids, dists, k, &sp, &ep, k, (uint32_t)i, d);
    }
}

/* search(::ParallelExhaustiveSearch, ctx, q, res)  (parallel-exhaustive.jl:64-102).
 * 1:n is cut into contiguous chunks of `minbatch` ids (Iterators.partition,
 * parallel.jl:612-614); each chunk fills its own KnnSorted(k); the chunks are
 * then pushed into the result IN BATCH ORDER (b = 1..nbatches), which is what
 * makes the result equal to the sequential one. */
void oracle_parallel_search(int metric, const void *db, int64_t dim, int64_t n,
                            const void *q, int32_t k, uint32_t *ids, float *dists,
                            int lanes, int64_t minbatch)
{
    if (minbatch < 1) minbatch = 1;
    int64_t nb = (n <= minbatch) ? 1 : (n + minbatch - 1) / minbatch;
    uint32_t *rids = (uint32_t *)calloc((size_t)(k * nb), sizeof(uint32_t));
    float *rd = (float *)calloc((size_t)(k * nb), sizeof(float));
    int32_t *used = (int32_t *)calloc((size_t)nb, sizeof(int32_t));
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t b = 0; b < nb; ++b) {
        int64_t s = (nb == 1) ? 1 : b * minbatch + 1;
        int64_t e = (nb == 1) ? n : ((b + 1) * minbatch < n ? (b + 1) * minbatch : n);
        int32_t sp = 1, ep = 0;
        for (int64_t i = s; i <= e; ++i) {
            float d = oracle_evaluate(metric, row_ptr(metric, db, dim, i - 1), q, dim, lanes);
            oracle_knnsorted_push(rids + b * k, rd + b * k, k, &sp, &ep, k, (uint32_t)i, d);
        }
        used[b] = ep - sp + 1;
    }
    int32_t sp = 1, ep = 0;
    for (int64_t b = 0; b < nb; ++b)
        for (int32_t j = 0; j < used[b]; ++j)
            oracle_knnsorted_push(ids, dists, k, &sp, &ep, k, rids[b * k + j], rd[b * k + j]);
    free(rids); free(rd); free(used);
}

/* searchbatch(index, ctx, Q, k)  (SimilaritySearch.jl:309-348).
 * index_kind 0 = ExhaustiveSearch (queries spread over threads, the
 * @BATCHES fan-out), 1 = ParallelExhaustiveSearch (each query split over
 * threads).  ids/dists are k x m column-major == m rows of k in C. */
void oracle_searchbatch(int metric, const void *db, int64_t dim, int64_t n,
                        const void *Q, int64_t m, int32_t k,
                        uint32_t *ids, float *dists, int lanes, int nthreads,
                        int index_kind, int64_t minbatch)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    for (int64_t j = 0; j < m * (int64_t)k; ++j) { ids[j] = 0; dists[j] = INFINITY; }
    if (index_kind == 1) {
        for (int64_t j = 0; j < m; ++j)
            oracle_parallel_search(metric, db, dim, n, row_ptr(metric, Q, dim, j), k,
                                   ids + j * k, dists + j * k, lanes, minbatch);
        return;
    }
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < m; ++j)
        oracle_search(metric, db, dim, n, row_ptr(metric, Q, dim, j), k,
                      ids + j * k, dists + j * k, lanes);
}

/* allknn!(index, ctx, ids, dists)  (allknn.jl:66-110): every object is
 * searched against the whole database, itself included. */
void oracle_allknn(int metric, const void *db, int64_t dim, int64_t n, int32_t k,
                   uint32_t *ids, float *dists, int lanes, int nthreads)
{
    oracle_searchbatch(metric, db, dim, n, db, n, k, ids, dists, lanes, nthreads, 0, 1);
}

/* allknn restricted to the object ids in `rows` (0-based), for sampled CPU
 * baselines: output row r holds the result for object rows[r]. */
void oracle_allknn_rows(int metric, const void *db, int64_t dim, int64_t n, int32_t k,
                        const int64_t *rows, int64_t nrows,
                        uint32_t *ids, float *dists, int lanes, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    for (int64_t j = 0; j < nrows * (int64_t)k; ++j) { ids[j] = 0; dists[j] = INFINITY; }
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < nrows; ++r)
        oracle_search(metric, db, dim, n, row_ptr(metric, db, dim, rows[r]), k,
                      ids + r * k, dists + r * k, lanes);
}

/* ------------------------------------------------------------------ */
/* FP64 gold standard: rank by (double distance, id).                  */
/* ------------------------------------------------------------------ */

typedef struct { double d; uint32_t id; } f64item;

static void f64_insert(f64item *buf, int32_t *len, int32_t k, double d, uint32_t id)
{
    if (*len == k) {
        f64item *last = &buf[k - 1];
        if (d > last->d || (d == last->d && id > last->id)) return;
        *len = k - 1;
    }
    int32_t i = *len;
    while (i > 0 && (buf[i - 1].d > d || (buf[i - 1].d == d && buf[i - 1].id > id))) {
        buf[i] = buf[i - 1];
        --i;
    }
    buf[i].d = d; buf[i].id = id;
    *len += 1;
}

void oracle_searchbatch_f64(int metric, const void *db, int64_t dim, int64_t n,
                            const void *Q, int64_t m, int32_t k,
                            uint32_t *ids, double *dists, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t j = 0; j < m; ++j) {
        f64item *buf = (f64item *)malloc(sizeof(f64item) * (size_t)k);
        int32_t len = 0;
        const void *q = row_ptr(metric, Q, dim, j);
        for (int64_t i = 0; i < n; ++i)
            f64_insert(buf, &len, k, oracle_evaluate_f64(metric, row_ptr(metric, db, dim, i), q, dim),
                       (uint32_t)(i + 1));
        for (int32_t t = 0; t < k; ++t) {
            ids[j * k + t] = t < len ? buf[t].id : 0;
            dists[j * k + t] = t < len ? buf[t].d : INFINITY;
        }
        free(buf);
    }
}

/* ------------------------------------------------------------------ */
/* rerank!(dist, db, q, ids, dists)  (rerank.jl:22-41).  The reference  */
/* sorts with sortperm; ties are ordered here by id so the result is    */
/* deterministic (the reference leaves the tie order to Base.sort).     */
/* ------------------------------------------------------------------ */

void oracle_rerank(int metric, const void *db, int64_t dim, const void *q,
                   uint32_t *ids, float *dists, int32_t len, int lanes)
{
    int32_t m = 0;
    for (int32_t i = 0; i < len; ++i) {
        if (ids[i] == 0) break;
        m = i + 1;
        dists[i] = oracle_evaluate(metric, row_ptr(metric, db, dim, ids[i] - 1), q, dim, lanes);
    }
    for (int32_t i = 1; i < m; ++i) { /* insertion sort by (dist, id) */
        float d = dists[i]; uint32_t id = ids[i];
        int32_t j = i;
        while (j > 0 && (dists[j - 1] > d || (dists[j - 1] == d && ids[j - 1] > id))) {
            dists[j] = dists[j - 1]; ids[j] = ids[j - 1]; --j;
        }
        dists[j] = d; ids[j] = id;
    }
}

/* ------------------------------------------------------------------ */
/* recallscore / macrorecall (perf.jl:31-33, 71-79).  gold and res are */
/* m columns of kg / kr ids; each column is cut to its first k.        */
/* ------------------------------------------------------------------ */

double oracle_macrorecall(const uint32_t *gold, int64_t kg, const uint32_t *res, int64_t kr,
                          int64_t m, int64_t k)
{
    double s = 0.0;
    for (int64_t j = 0; j < m; ++j) {
        const uint32_t *g = gold + j * kg, *r = res + j * kr;
        /* |Set(g[1:k]) ∩ Set(r[1:k])| / k */
        int64_t hit = 0, gl = 0;
        for (int64_t a = 0; a < k; ++a) {
            int dup = 0;
            for (int64_t b = 0; b < a; ++b) if (g[b] == g[a]) { dup = 1; break; }
            if (dup) continue;
            for (int64_t b = 0; b < k; ++b) {
                int dup2 = 0;
                for (int64_t c = 0; c < b; ++c) if (r[c] == r[b]) { dup2 = 1; break; }
                if (!dup2 && r[b] == g[a]) { ++hit; break; }
            }
            ++gl;
        }
        (void)gl;
        s += (double)hit / (double)k;
    }
    return s / (double)m;
}

/* bitsketch(R, X) (src/proj/bitsketches.jl:101-104 via _bitsketch_apply,
 * :56-57): transform (src/proj/Projections.jl:137-143: coordinate c of row r
 * is dot32(R column c, x_r)), then packsigns (bitsketches.jl:19-32: bit c of
 * word c / 64 set iff the coordinate is >= 0, unused high bits 0).  R is
 * given as outdim rows of indim (the bytes of the Julia (indim, outdim)
 * matrix); out is n rows of ceil(outdim / 64) words. */
void oracle_bitsketch(const float *R, int64_t indim, int64_t outdim, const float *X, int64_t n,
                      uint64_t *out, int lanes)
{
    const int64_t words = (outdim + 63) / 64;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t r = 0; r < n; ++r) {
        uint64_t *o = out + r * words;
        for (int64_t w = 0; w < words; ++w) o[w] = 0;
        for (int64_t c = 0; c < outdim; ++c)
            if (dot32(R + c * indim, X + r * indim, indim, lanes) >= 0.0f) o[c >> 6] |= (uint64_t)1 << (c & 63);
    }
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
