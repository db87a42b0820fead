// kernels.h -- host-side launchers of the device kernels (internal to libssgpu).
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

namespace ssg {

enum Metric { SQL2 = 0, L2 = 1, NORMCOSINE = 2, COSINE = 3, IP = 4, HAMMING = 5 };

// A scan over database rows [0, n) for m queries.  Each (query, split) pair
// leaves its `kk` smallest keys, sorted ascending, in
// cand[(q * splits + s) * kk + i]; empty slots hold KEY_EMPTY.
struct ScanArgs {
    int metric;
    int64_t n;         // database rows
    int64_t dim;       // floats per row (float metrics) or words (Hamming)
    int64_t m;         // queries
    int kk;            // keys kept per (query, split)
    int splits;        // database splits
    int64_t split_len; // rows per split (last may be shorter)
    uint64_t *cand;    // m * splits * kk keys
    uint64_t *gheap;   // global heap storage when kk is too large for shared memory
    int64_t id_base;   // added to every 0-based row id in the keys
    // optional per-query bound shared by all splits (float_to_ordered of a
    // distance, all ones = none yet): every heap that holds kk keys lowers it
    // to its frontier, and every heap filters against it -- any heap's kk-th
    // key bounds the query's kk-th key over all splits, so the merged
    // candidates do not change
    uint32_t *qbound = nullptr;
};

// Exact FP32 scan: difference form for SqL2/L2, sequential-FMA dot for the
// others, summed in index order (bit-identical to the oracle's lanes=1 sum).
cudaError_t launch_direct_f32(const ScanArgs &a, const float *db, const float *db_norm,
                              const float *q, const float *q_norm, cudaStream_t st, int *launches);

// Hamming scan over packed UInt64 sketches.
cudaError_t launch_hamming(const ScanArgs &a, const uint64_t *db, const uint64_t *q,
                           cudaStream_t st, int *launches);

// Global-heap bytes a scan needs (0 when its heaps fit in shared memory).
size_t direct_gheap_bytes(const ScanArgs &a);
size_t hamming_gheap_bytes(const ScanArgs &a);

// Merges the `segs` sorted key lists of every query and writes the k
// outputs: 1-based ids and distances, 0 / +Inf when empty.  With
// exclude_self, query j is object j + self_base and is dropped from its list
// (the list holds k+1 keys then).
struct FinalizeArgs {
    const uint64_t *cand;
    int segs;
    int kk;
    int64_t m;
    int k_out;
    int exclude_self;
    int64_t self_base;
    uint32_t *out_ids;
    float *out_dists;
    // optional: per-query object ids for exclude_self (overrides self_base)
    const int64_t *self_ids = nullptr;
    // optional completeness check of an approximate candidate list: flags[j]
    // = 1 (and *flag_count += 1) when the kk approximate candidates do not
    // provably contain the exact top (k + exclude_self).  1: GEMM-form keys
    // of SqL2 / L2 (|x|^2 - 2 x.q), error err_scale (|x|max + |q|)^2; 2:
    // dot-product keys (-x.q), error err_scale |x|max |q|.
    int check = 0;
    const float *q_sq = nullptr;   // |q|^2 per query
    float max_x_sq = 0.0f;         // max |x|^2 over the database (the metric's rows as stored)
    float err_scale = 0.0f;        // the error bound's scale (see the check's kinds above)
    int64_t n_total = 0;           // database rows
    int *flags = nullptr;
    int *flag_count = nullptr;
    // rows of the database the keys index: a key with a larger id is treated
    // as empty instead of being read (the rerank kernels set it always)
    int64_t n_rows = 0;
    // candidates re-ranked per query, from the merged segments (0: kk, the
    // segment length).  More than kk when each heap kept only part of the
    // list (the plain method's half heaps on the tensor cores).
    int rerank = 0;
};
cudaError_t launch_finalize(const FinalizeArgs &a, cudaStream_t st, int *launches);

// Keys one merge block sorts at most (64 KB of shared memory).
constexpr int kMergeKeys = 8192;
// One reduction pass: each group of `group` sorted kk-key segments of every
// query -> one sorted segment of its kk smallest keys (ceil(segs/group) out).
cudaError_t launch_merge_groups(const uint64_t *in, int64_t m, int segs, int kk, int group, uint64_t *out,
                                cudaStream_t st, int *launches);

// Row norms: out[i] = sqrt(sum x^2) (COSINE) in sequential FMA order.
cudaError_t launch_row_norms(const float *x, int64_t rows, int64_t dim, float *out,
                             cudaStream_t st, int *launches);

// Element casts to Float32 (CastF32 twins): elem is SSG_ELEM_*.
cudaError_t launch_cast_f32(const void *src, int elem, int64_t count, float *dst,
                            cudaStream_t st, int *launches);

// Exact rerank of candidate id lists (rerank!): per query j, ids[j*len ..]
// (1-based, 0 terminates) are re-scored and sorted by (distance, id).
// db / q are float rows (float metrics) or UInt64 words (HAMMING); norms are
// used by COSINE only.
cudaError_t launch_rerank(int metric, const void *db, const float *db_norm, int64_t dim,
                          const void *q, const float *q_norm, int64_t m, int len,
                          uint32_t *ids, float *dists, cudaStream_t st, int *launches);

// ---- BF16 tensor-core path (tc_bf16.cu) ----
// Queries / database rows as BF16 tiles of 128 rows in the swizzled tcgen05
// operand layout (K padded to a multiple of 32).
int tc_padded_k(int64_t dim);
int64_t tc_tiles(int64_t rows);
size_t tc_tile_bytes(int64_t dim);
// Chooses query tiles per CTA and pipeline depth; false if kk cannot fit.
bool tc_choose(int kp, int kk, int *qt, int *stages);
// Whether the wide scan's heaps and ring fit for this K and candidate count
// (one CTA, or a CTA pair with half-size ring stages).
bool tc_wide_fits(int kp, int kk);
// Ring stages of the wide scan at this K and candidate count (0: it does not fit).
int tc_wide_stages(int kp, int kk);
bool tc_pair_fits(int kp, int kk);
// Sorted candidate segments the scan writes per (query, split) for a CTA with
// `qt` query tiles (the epilogue splits a tile's columns between warps).
int tc_segments_per_split(int qt);
// With a map, tile row i holds source row map[i].  split: 0 = BF16 rows
// (K = kp); 1 = database rows of the two-piece plain method, [hi | lo | hi];
// 2 = its query rows, [hi | hi | lo] (K = 3 kp; see bf16_tile_kernel).
cudaError_t launch_bf16_tiles(const float *x, int64_t rows, int64_t dim, int64_t tiles, uint8_t *out,
                              cudaStream_t st, int *launches, const uint32_t *map = nullptr, int split = 0);
// |x|^2 (SqL2/L2) or 1/|x| (Cosine) per padded row (of source row map[i]
// with a map).
cudaError_t launch_tc_norms(int metric, const float *x, int64_t rows, int64_t dim, int64_t padded, float *out,
                            cudaStream_t st, int *launches, const uint32_t *map = nullptr);
// The fused scan: per (query, split) the kk best approximate keys.  *err is
// set non-zero if a bounded wait gave up.  wide: 256-row database tiles per
// MMA when the heaps leave room for its ring (d_tiles then must hold an even
// number of tiles, as every tile set of the library does).  With perm / rot (allknn over
// tiles built in a locality order, one launch for all queries): perm[p] is
// the id of the row at position p of both tile sets, query CTA x starts at
// database tile rot[x], keys carry ids and each query's candidates go to
// the row of its id.  wave > 0: the wide scan is launched `wave` query tiles
// at a time.  pair (with wide): the scan runs on CTA pairs with M = 256 MMAs
// (the query tile set must then hold an even number of tiles).  qbound: m
// words set to all ones, the per-query bound every heap of a query shares
// (see ScanArgs::qbound).
cudaError_t launch_tc_scan(int metric, const uint8_t *q_tiles, const uint8_t *d_tiles, const float *d_norm,
                           int64_t n, int64_t m, int64_t dim, int kk, int splits, uint64_t *cand, int *err,
                           cudaStream_t st, int *launches, int *qt_out, const uint32_t *perm = nullptr,
                           const int *rot = nullptr, bool wide = false, int64_t wave = 0, bool pair = false,
                           uint32_t *qbound = nullptr);
// The same scan for candidate lists too long for the two heaps per query of
// the wide and pair scans: CTA pairs with one heap per query (one segment per
// split and query).  tc_long_fits tells whether kk fits.
bool tc_long_fits(int kp, int kk);
cudaError_t launch_tc_scan_long(int metric, const uint8_t *q_tiles, const uint8_t *d_tiles, const float *d_norm,
                                int64_t n, int64_t m, int64_t dim, int kk, int splits, uint64_t *cand, int *err,
                                cudaStream_t st, int *launches, const uint32_t *perm, const int *rot, int64_t wave,
                                uint32_t *qbound);
// Locality order from a kk = 1 scan of n rows against P pivots (cand: n x
// segs keys): pivot[i] (the bucket: rank[pivot], or the pivot itself with
// rank null), bucket counts / starts, perm (position -> row, rows grouped by
// bucket) and rot (start tile of each query tile's scan: its first row's
// group).
cudaError_t launch_locality_order(const uint64_t *cand, int64_t n, int segs, int P, const uint32_t *rank,
                                  uint32_t *pivot, int *count, int *start, int *cursor, uint32_t *perm, int *rot,
                                  cudaStream_t st, int *launches);
// Threshold-filter scan for candidate counts beyond the on-chip heaps: every
// (query, row) with d~ <= thr[query] is appended to the query's fcap-key list.
cudaError_t launch_tc_filter(int metric, const uint8_t *q_tiles, const uint8_t *d_tiles, const float *d_norm,
                             int64_t n, int64_t m, int64_t dim, int splits, const float *thr, uint64_t *fout,
                             int *fcount, int fcap, int *err, cudaStream_t st, int *launches);
// thr[q] = min over segments of the segment's kk-th key distance.
cudaError_t launch_sample_bound(const uint64_t *cand, int64_t m, int segs, int kk, float *thr, cudaStream_t st,
                                int *launches);
// Sorted first kk filtered keys per query; short or overflowed lists flagged.
cudaError_t launch_filter_select(const uint64_t *fout, const int *fcount, int64_t m, int fcap, int kk,
                                 uint64_t *cand, int *flags, int *flag_count, cudaStream_t st, int *launches);
// Merge + exact FP32 rerank of the candidates + (distance, id) sort + decode.
cudaError_t launch_finalize_rerank(int metric, const FinalizeArgs &f, const float *db, const float *db_norm,
                                   int64_t dim, const float *q, const float *q_norm, cudaStream_t st,
                                   int *launches);

// ---- K-streaming tensor-core path for any dimension, BF16 or FP8 (tc_stream.cu) ----
int stream_kbytes(int64_t dim, int fp8);          // padded bytes per row
size_t stream_tile_bytes(int64_t dim, int fp8);   // bytes per 128-row tile
constexpr int kBoundWords = 16;                   // shared pruning-bound words per query
int stream_heap_rows(int64_t m);                  // query rows of a tile that own heaps
bool stream_choose(int kk, int heap_rows, int *cs, int *stages);
// rows -> K-block tiles; FP8 also writes the per-row scale (scale may be null
// for BF16).  split 1 / 2 (BF16): the plain method's two-piece tiles, K = 3 x
// the padded dim, database / query layout (tc_stream.cu)
cudaError_t launch_stream_tiles(const float *x, int64_t rows, int64_t dim, int fp8, int64_t tiles, uint8_t *out,
                                float *scale, cudaStream_t st, int *launches, int split = 0);
// per padded database row: alpha / beta of the approximate distance
cudaError_t launch_stream_coefs(int metric, const float *x, int64_t rows, int64_t dim, int64_t padded,
                                const float *scale, float *alpha, float *beta, cudaStream_t st, int *launches);
cudaError_t launch_stream_scan(const uint8_t *q_tiles, const uint8_t *d_tiles, const float *alpha, const float *beta,
                               const float *qgamma, int64_t n, int64_t m, int64_t dim, int fp8, int kk, int splits,
                               int heap_rows, uint32_t *gbound, uint64_t *cand, int *err, cudaStream_t st,
                               int *launches, int *segs_per_split);

// ---- plain FP32 GEMM-form scan (gemm_f32.cu) ----
// Writes `splits` sorted segments of kk keys per query.
bool gemm_fits(int kk);
int gemm_ctas_per_sm(int kk);
// k-major tiles of 128 rows (dim-major, zero-padded to gemm_kpad(dim)).
int gemm_kpad(int64_t dim);
size_t gemm_tile_floats(int64_t dim);
cudaError_t launch_gemm_tiles(const float *x, int64_t rows, int64_t dim, int64_t tiles, float *out, cudaStream_t st,
                              int *launches);
// Sign bit sketches of n rows against outdim projection rows, from k-major
// tiles of both (out: n rows of ceil(outdim / 64) words).
cudaError_t launch_bitsketch(const float *xtiles, const float *rtiles, int64_t dim, int64_t n, int64_t outdim,
                             uint64_t *out, cudaStream_t st, int *launches);
// a.split_len must be a multiple of 128 (tile-aligned splits).
cudaError_t launch_gemm_f32(const ScanArgs &a, const float *dtiles, const float *xaux, const float *qtiles,
                            const float *q_norm, cudaStream_t st, int *launches);

// ---- closest pairs (direct.cu) ----
// keys[j * kk + t] = (dists[j][t], j * kk + t), empty where ids[j][t] == 0
cudaError_t launch_pair_keys(const uint32_t *ids, const float *dists, int64_t total, uint64_t *keys, cudaStream_t st,
                             int *launches);
// (i, j, d) of the merged top k: i = ids[flat], j = flat / kk + 1
cudaError_t launch_pair_decode(const uint32_t *sel_ids, const float *sel_d, int k, const uint32_t *ids, int kk,
                               int32_t *oi, int32_t *oj, float *od, cudaStream_t st, int *launches);

// ---- helpers (direct.cu) ----
// out[i] = sum x^2 per row (sequential FMA) and *max_out = max over rows
// (max_out must be zeroed first).
cudaError_t launch_row_sq_norms(const float *x, int64_t rows, int64_t dim, float *out, float *max_out,
                                cudaStream_t st, int *launches);
// dst row i = src row idx[i] (rows of row_bytes bytes, a multiple of 4).
cudaError_t launch_gather_rows(const void *src, const int64_t *idx, int64_t count, size_t row_bytes, void *dst,
                               cudaStream_t st, int *launches);
// ids/dists row idx[i] (k entries) = src row i.
cudaError_t launch_scatter_results(const uint32_t *src_ids, const float *src_d, const int64_t *idx, int64_t count,
                                   int k, uint32_t *ids, float *dists, cudaStream_t st, int *launches);

int device_sm_count();

// ---- learned shortlist (mlp.cu, learned.cu) ----
// C (M x N, row-major, row stride ldc) = A B^T on the tensor cores, A = M x K
// and B = N x K given K-major (X[r * ld + k]) or transposed (X[k * ld + r]),
// FP32 in memory, BF16 operands, FP32 accumulation.  Epilogue: + bias[n],
// ReLU, * (mask[m * ldc + n] > 0), per-M-tile column sums
// colsum[tile * N + n].  splits > 1 splits K: part s is written at
// C + s * M * ldc (no epilogue then).  exact: operands as three BF16 pieces
// and six piece products (FP32-class accuracy, ~2^-24).  *err receives a
// non-zero code if a bounded wait gave up.
struct MlpGemm {
    const float *A = nullptr;
    int64_t lda = 0;
    int a_kmajor = 1;
    const float *B = nullptr;
    int64_t ldb = 0;
    int b_kmajor = 1;
    float *C = nullptr;
    int64_t ldc = 0;
    int M = 0, N = 0, K = 0;
    int splits = 1;
    const float *bias = nullptr;
    int relu = 0;
    const float *mask = nullptr;
    float *colsum = nullptr;
    int exact = 0;
    int *err = nullptr;
};
cudaError_t mlp_gemm(const MlpGemm &g, cudaStream_t st, int *launches);
int mlp_gemm_mtiles(int M);  // M tiles = rows of the column-sum partials
int mlp_gemm_ntiles(int N);  // N tiles of a product with N columns
// K splits giving about `want` CTAs for a product of `ctas` output tiles (at
// most one split per 64-element K-block, the K-blocks spread evenly)
int mlp_splits(int K, int ctas, int want);
// C (M x N) = sum of the `parts` split products P[p] (M x N each) + bias[n], ReLU
cudaError_t mlp_reduce_parts(const float *P, int parts, int M, int N, const float *bias, int relu, float *C,
                             cudaStream_t st, int *launches);
cudaError_t mlp_triplet(const float *Z, int B, int E, float margin, float *dZ, float *loss_sum, int *active,
                        cudaStream_t st, int *launches);
// out[p * N + n] = sum of G[r][n] over the p-th of `parts` row ranges
cudaError_t mlp_colsum_parts(const float *G, int rows, int N, int parts, float *out, cudaStream_t st, int *launches);
// out[i] = sum over p < parts of G[p * count + i]
cudaError_t mlp_sum_parts(const float *G, int parts, int64_t count, float *out, cudaStream_t st, int *launches);
// Adam steps on four parameter groups in one launch (group g: W[g], its
// gradient summed from parts[g] partials of count[g] entries, moments M, V)
cudaError_t mlp_adam4(float *const W[4], const float *const G[4], const int parts[4], float *const M[4],
                      float *const V[4], const int64_t count[4], float lr, int step, cudaStream_t st, int *launches);
// X = [S[idx[off..]]; S[idx[T + off..]]; S[idx[2T + off..]]] (bb rows each)
cudaError_t mlp_gather3(const float *S, const int64_t *idx, int64_t T, int64_t off, int bb, int d, float *X,
                        cudaStream_t st, int *launches);

// What the learned code needs of an index.
struct IndexView {
    const float *db;
    const float *db_norm;
    int64_t n, dim;
    int metric;
    cudaStream_t stream;
    int *launches;
};
struct TrainArgs {
    int64_t sample, triplets;
    int epochs;
    int64_t hidden, out_dim;
    int batch;
    float lr, margin;
    uint64_t seed;
    int shortlist;
    // fraction of negatives drawn from the anchor's exact neighbours just
    // beyond the positives (ranks 11..50 in the sample), the rest uniform
    float hard;
};
struct LearnedModel;
void learned_free(LearnedModel *m);
double learned_get(const LearnedModel *m, const char *key, bool *found);
bool learned_set(LearnedModel *m, const char *key, double v);
int learned_train(const IndexView &v, const TrainArgs &t, LearnedModel **out, std::string &err);
int learned_index_db(LearnedModel *m, const IndexView &v, std::string &err);
int learned_search(LearnedModel *m, const IndexView &v, const float *dq, const float *dqn, int64_t mq, int k,
                   uint32_t *d_ids, float *d_dists, std::string &err);
int learned_save(const LearnedModel *m, const char *path, std::string &err);
int learned_load(const IndexView &v, const char *path, LearnedModel **out, std::string &err);
void learned_set_recall(LearnedModel *m, double r);
int learned_grad_check(int64_t d, int64_t H, int64_t E, const float *W1, const float *b1, const float *W2,
                       const float *b2, const float *X, int B, float margin, float *loss, float *gW1, float *gb1,
                       float *gW2, float *gb2, std::string &err);

// Records `msg` as the calling thread's last error (what ssg_last_error(NULL,
// ...) returns) and returns `code`.
int report_error(int code, const char *msg);

}  // namespace ssg
