/*
 * ssgpu.h -- C ABI of libssgpu.so, the GB300 exhaustive k-NN engine behind
 * SimilaritySearch.jl's `searchbatch` / `allknn` path.
 *
 * Every entry point takes plain pointers and sizes; nothing crosses the
 * boundary but C types.  Each call returns SSG_OK (0) or a negative status and
 * never aborts; the text of the last failure is kept per index (or per thread
 * for failures without an index) and read with ssg_last_error.
 *
 * Layout.  A Julia `Matrix{Float32}(d, n)` (column i = object i) is, byte for
 * byte, a C row-major n x d array, so databases and query sets are passed as
 * `n` rows of `ld` elements (ld >= dim, the column stride of a Julia view).
 * Sketch databases (`Matrix{UInt64}(W, n)`) are n rows of W words.  Result
 * matrices `(k, m)` are m rows of k: ids are 1-based UInt32, unfilled slots
 * hold id 0 and +Inf, and every row is sorted by (distance, id), the order
 * `KnnSorted` produces (src/pqueue/knnsorted.jl:68-101,140-168).
 *
 * Threading.  One handle owns one CUDA stream and a mutex: calls on a handle
 * are serialised, distinct handles may be used from different threads.
 */
#ifndef SSGPU_H
#define SSGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define SSG_OK            0
#define SSG_EINVAL       -1   /* bad argument: shapes, empty inputs, k out of range */
#define SSG_ENOMEM       -2   /* device or pinned-host allocation failed            */
#define SSG_ECUDA        -3   /* a CUDA runtime / kernel error                      */
#define SSG_ETIMEOUT     -4   /* a bounded device-side wait gave up                 */
#define SSG_EUNSUPPORTED -5   /* metric / element type / mode not supported         */

/* ---- distances (SimilaritySearch.jl `Dist.*`) ----
 * SQL2        Dist.SqL2        sum (x_i - q_i)^2            src/dist/vecs.jl:86,93-102
 * L2          Dist.L2          sqrt(sum (x_i - q_i)^2)      src/dist/vecs.jl:52,59-67
 * NORMCOSINE  Dist.NormCosine  1 - sum x_i q_i              src/dist/cos.jl:39,76-84
 * COSINE      Dist.Cosine      1 - x.q / (|x| |q|)          src/dist/cos.jl:16,103
 * IP          (new)            -sum x_i q_i  (NormCosine - 1, max inner product)
 * HAMMING     Dist.Bits.Hamming  Float32(sum popcount(x_w xor q_w))  src/dist/bits.jl:10,18-25
 * The Dist.CastF32 twins (src/dist/vecs-cast-f32.jl:76-93,148-189) are the
 * float metrics over a non-Float32 element type: pass that element type and
 * the library casts every element to Float32 on upload. */
#define SSG_METRIC_SQL2        0
#define SSG_METRIC_L2          1
#define SSG_METRIC_NORMCOSINE  2
#define SSG_METRIC_COSINE      3
#define SSG_METRIC_IP          4
#define SSG_METRIC_HAMMING     5

/* ---- element types of host buffers ---- */
#define SSG_ELEM_F32  0
#define SSG_ELEM_U64  1   /* packed bit sketches, HAMMING only */
#define SSG_ELEM_F64  2   /* CastF32 twins: cast to Float32 on upload */
#define SSG_ELEM_F16  3
#define SSG_ELEM_U8   4
#define SSG_ELEM_I8   5

/* ---- precision modes of the float metrics ----
 * FP32: the plain method; results match ExhaustiveSearch on the same inputs
 *       (distances within 1e-5 relative, ids equal outside near-tie bands).
 * BF16: BF16 tensor-core distances over-fetching c*k candidates per query,
 *       re-ranked in exact FP32 difference form (c = "overfetch" param).
 * FP8:  FP8 e4m3 with a per-vector scale, same over-fetch and FP32 rerank. */
#define SSG_PREC_FP32  0
#define SSG_PREC_BF16  1
#define SSG_PREC_FP8   2

typedef struct ssg_index ssg_index;

/* Builds a GPU index over `n` objects of `dim` elements (row stride `ld`)
 * copied from host memory.  Replaces the construction of
 * ExhaustiveSearch(dist, MatrixDatabase(X)) / ParallelExhaustiveSearch
 * (src/exact/sequential-exhaustive.jl:18-21, src/exact/parallel-exhaustive.jl:26-29).
 * For HAMMING, `dim` is the number of UInt64 words per sketch. */
int ssg_create(int metric, int elem_type, int64_t dim, int64_t n,
               const void *host_db, int64_t ld, int precision_mode, ssg_index **out);

/* Same, from a database already in device memory (n rows of `ld` elements of
 * `elem_type`); the library keeps its own copy. */
int ssg_create_device(int metric, int elem_type, int64_t dim, int64_t n,
                      const void *dev_db, int64_t ld, int precision_mode, ssg_index **out);

/* Same, from a MMapMatrixDatabase file (src/db/mmapmatrixdatabase.jl:10-27,
 * 151-175): a 4096-byte header (magic 0x4D4D444231000001, version 1, dim,
 * element type code, n) followed by the column-major data, which streams
 * from the mapped file into device memory (no host copy of the whole file).
 * Element types: Float32, Float64, Float16, Int8, UInt8 (cast to Float32 for
 * the float metrics, as the CastF32 twins do) and UInt64 (HAMMING). */
int ssg_create_mmap(int metric, const char *path, int precision_mode, ssg_index **out);

/* k nearest neighbours of `m` queries (host rows of `dim` elements of the
 * index's element type, contiguous) written to host out_ids / out_dists
 * (m rows of k).  Replaces the matrix searchbatch! loop
 * (src/SimilaritySearch.jl:331-348) over search(::ExhaustiveSearch)
 * (src/exact/sequential-exhaustive.jl:68-80) and
 * search(::ParallelExhaustiveSearch) (src/exact/parallel-exhaustive.jl:64-102).
 * flags: reserved, pass 0. */
int ssg_search(ssg_index *idx, const void *host_q, int64_t dim, int64_t m, int32_t k,
               uint32_t *out_ids, float *out_dists, int32_t flags);

/* Same as ssg_search with queries and results in device memory (results are
 * written on the index's stream; the call returns once they are complete). */
int ssg_search_device(ssg_index *idx, const void *dev_q, int64_t m, int32_t k,
                      uint32_t *dev_ids, float *dev_dists, int32_t flags);

/* Runs nb query batches of different sizes and k as one search: batch b has
 * m[b] queries at dev_q[b] (device rows of dim elements of the index's type)
 * and receives m[b] rows of k[b] results at dev_ids[b] / dev_dists[b] (device
 * memory).  The arrays themselves are host arrays of nb entries.  Batches of
 * the same k share the query tiles and one scan of the database (one scan per
 * distinct k), so each batch's rows are those of a separate call with its k.
 * Batches with m[b] == 0 are skipped.  Replaces per-request searchbatch!
 * calls on a request stream.  With the reduced-precision scans the device
 * work of each k's search is replayed from a CUDA graph when its shape
 * (queries rounded up to 32, k) repeats ("graphs" param, default 1;
 * "graph_replays", "last_graph" readable). */
int ssg_search_batches(ssg_index *idx, int32_t nb, const void *const *dev_q, const int64_t *m,
                       const int32_t *k, uint32_t *const *dev_ids, float *const *dev_dists);

/* All-vs-all k-NN over the indexed objects.  exclude_self == 0 keeps each
 * object in its own result like allknn! (src/allknn.jl:66-110); exclude_self
 * != 0 computes k+1 neighbours and drops the object itself (or the last one
 * when the object is not among them).  Results are n rows of k. */
int ssg_allknn(ssg_index *idx, int32_t k, int32_t exclude_self,
               uint32_t *out_ids, float *out_dists);
int ssg_allknn_device(ssg_index *idx, int32_t k, int32_t exclude_self,
                      uint32_t *dev_ids, float *dev_dists);

/* Appends `count` objects (host rows of `dim` elements, contiguous) with ids
 * n+1 .. n+count.  Replaces append_items! / push_item!
 * (src/exact/sequential-exhaustive.jl:33-47). */
int ssg_append(ssg_index *idx, const void *host_rows, int64_t count);

/* Re-scores and sorts candidate lists exactly (rerank!, src/rerank.jl:22-86):
 * row j of ids (len entries, 1-based, 0 ends the list) is re-evaluated
 * against query j with the index's metric in FP32 and sorted by
 * (distance, id).  Host buffers; m rows. */
int ssg_rerank(ssg_index *idx, const void *host_q, int64_t m, int32_t len,
               uint32_t *ids, float *dists);

/* Tunables: "overfetch" (candidates per k in BF16/FP8 modes), "splits"
 * (database splits per query tile, 0 = auto), "margin" (extra candidates of
 * the plain GEMM-form scan, 0 = auto), "exact_scan" (1 = plain method through
 * the direct difference-form scan only), "plain" (1 = plain FP32 method on a
 * BF16/FP8 index, e.g. to calibrate "overfetch" against it), "profile"
 * (1 = time the scan kernel with events), "graphs" (0 = no CUDA-graph replay
 * in ssg_search_batches), "wide" (0 = BF16 scans in 128 x 128 tiles instead
 * of 128 x 256), "pair" (1 = BF16 / split scans on CTA pairs with M = 256
 * MMAs), "long_lists" (0 = BF16 candidate lists too long for two heaps per
 * query go through the threshold filter instead of CTA pairs with one heap
 * per query; same candidates), "locality" (0 = BF16 allknn scans in id order
 * instead of the pivot-grouped order; results are identical either way),
 * "locality_rows" (database rows per pivot of that order, 64..65536, default
 * 128), "locality_chain" (0 = the pivots' groups in pivot order instead of a
 * greedy nearest-pivot chain; results identical), "plain_tc"
 * (0 = keep the plain method on the CUDA cores; by default the float
 * metrics over at least 4096 objects run it on the tensor cores: a two-piece BF16 scan -- query tiles resident for
 * dim <= 128, both operands streamed along K beyond -- whose candidates are
 * re-scored in exact FP32 and certified complete, uncertified queries
 * recomputed by the exact scan; results identical either way).  Unknown
 * keys return SSG_EINVAL. */
int ssg_set_param(ssg_index *idx, const char *key, double value);
/* Readable keys: the tunables plus "n", "dim", "metric", "precision",
 * "main_kernel_ms" / "main_kernel_launches" (accumulated while profiling),
 * "kernel_launches" (kernels launched by the last call), "fallbacks" (queries
 * the last plain call recomputed with the exact scan), "last_plain_tc"
 * (1 when the last plain call ran on the tensor cores), "max_x_sq",
 * "device_bytes". */
int ssg_get_param(ssg_index *idx, const char *key, double *value);

/* Runs the index's work on `stream` (a cudaStream_t) instead of its own. */
int ssg_set_stream(ssg_index *idx, void *stream);

/* Copies the last error text (NUL terminated, truncated to len). idx may be
 * NULL for failures of ssg_create*. Returns the full length of the text. */
int ssg_last_error(ssg_index *idx, char *buf, int64_t len);

/* Releases the index and its device memory. */
void ssg_destroy(ssg_index *idx);

/* ABI version (major * 10000 + minor * 100 + patch). */
int ssg_version(void);

/* ---- learned shortlist (no counterpart in the reference) ----
 * ssg_train_mlp trains a network d -> hidden (ReLU) -> out_dim on the index's
 * own data: a seeded sample of `sample_n` objects, their exact 50 nearest
 * neighbours within the sample (this library's allknn), `triplets` triplets
 * (anchor; one of its 10 nearest as the positive; as the negative, with
 * probability "train_hard" (default 0.5) one of its neighbours ranked 11..50,
 * else a uniform object of the sample) and the triplet loss
 * max(0, |f(a)-f(p)|^2 - |f(a)-f(n)|^2 + 1), minimised with Adam (learning
 * rate `lr`) for `epochs` passes in mini-batches of `batch`; every product
 * on the tensor cores with BF16 operands, FP32 accumulation and FP32 master
 * weights.  hidden == 0 gives a
 * seeded Gaussian random projection d -> out_dim and no training: the
 * baseline the network is measured against.  The database is then embedded
 * and indexed.  From then on ssg_search / ssg_search_device shortlist the
 * "shortlist" (default 512) nearest embeddings, re-score them with the exact
 * FP32 distance of the index's metric and return the k best -- but only
 * while "learned_recall" (recall@10 of that pipeline against the plain
 * method, measured on 256 database objects when the model is trained or
 * loaded) is at least "learned_target" (default 0.99) and "learned" is 1;
 * otherwise the index's own method answers.  "learned_used" tells whether the
 * last search took the learned path.  Float metrics only; 1 <= out_dim <= 256,
 * hidden <= 8192.
 * Readable keys: "learned_recall", "learned_ready", "train_loss",
 * "train_seconds", "train_steps", "shortlist", "train_hard". */
int ssg_train_mlp(ssg_index *idx, int64_t sample_n, int64_t triplets, int32_t epochs,
                  int32_t hidden, int32_t out_dim, int32_t batch, double lr, uint64_t seed);
/* Model files: "SSGMLP01", int64 d, hidden, out_dim, then the FP32 weights
 * W1 (hidden x d), b1, W2 (out_dim x hidden), b2 (W1 = out_dim x d alone when
 * hidden == 0).  Loading embeds and indexes the database again. */
int ssg_save_model(ssg_index *idx, const char *path);
int ssg_load_model(ssg_index *idx, const char *path);
/* One forward + backward pass of the network on a host batch X of 3*batch
 * rows (anchors, positives, negatives) with host weights, through the
 * training step's tensor-core kernels with each operand carried as three BF16
 * pieces (FP32-class accuracy); writes the mean triplet loss (margin
 * `margin`) and the weight gradients to host buffers.  For testing the
 * training kernels against a CPU reference. */
int ssg_mlp_grad_check(int64_t d, int64_t hidden, int64_t out_dim, const float *W1,
                       const float *b1, const float *W2, const float *b2, const float *X,
                       int32_t batch, float margin, float *loss, float *gW1, float *gb1,
                       float *gW2, float *gb2);

/* The k closest pairs (i, j) between the indexed objects (i) and the m
 * objects of host_B (j; rows of dim elements of the index's type), or among
 * the indexed objects themselves when host_B is NULL (m is then ignored):
 * bichromatic_kclosestpairs / closestpairs / closestpair
 * (src/bichromatic/bichromaticclosestpairs.jl, closestpairs.jl,
 * closestpair.jl).  Each object of B takes its min_k (>= k) nearest indexed
 * objects -- itself excluded when samedata != 0 (always with host_B NULL),
 * i.e. when object j of B is indexed object j -- and the k smallest
 * candidates overall are returned sorted by (distance, j, rank within j),
 * 1-based ids; *count receives how many exist (< k when there are fewer
 * pairs; the rest of the outputs are 0 / +Inf).  Outputs are host arrays of
 * k entries. */
int ssg_closestpairs(ssg_index *idx, const void *host_B, int64_t m, int32_t k, int32_t min_k,
                     int32_t samedata, int32_t *out_i, int32_t *out_j, float *out_d, int64_t *count);

/* Bit sketches (bitsketch(R, X), src/proj/bitsketches.jl:19-32,56-57,101-104
 * over transform, src/proj/Projections.jl:137-143): for each of the n rows x
 * of dev_X (n rows of dim Float32) and each of the outdim projection rows r
 * of dev_R (outdim rows of dim Float32: the bytes of the Julia (dim, outdim)
 * map), bit c of the row's sketch is 1 iff dot(r_c, x) >= 0, packed 64 per
 * UInt64 word (coordinate c in bit c % 64 of word c / 64, unused high bits
 * 0) into dev_out (n rows of ceil(outdim / 64) words): the C3 sketches the
 * Hamming scan searches.  The dot products are the sequential FP32 fma
 * chain.  Device buffers; work on `stream` (cudaStream_t, NULL = default),
 * the call returns when it is done. */
int ssg_bitsketch(const void *dev_R, int64_t dim, int64_t outdim, const void *dev_X, int64_t n,
                  uint64_t *dev_out, void *stream);

/* Exact k-NN that allocates no device memory.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc -- programs
 * whose own allocator already owns the GPU's memory, and request paths that
 * must not allocate because cudaMalloc can synchronise the device.
 * Database (n rows of dim Float32, or dim UInt64 words for HAMMING), queries
 * (m rows) and results (m rows of k: 1-based ids, distances; 0 / +Inf when
 * empty; (distance, id) order) are caller-owned device memory.  Metrics:
 * SQL2, L2, NORMCOSINE, IP, HAMMING (COSINE returns SSG_EUNSUPPORTED).
 * Results are those of ssg_search_device on the same data in the plain
 * method.  The candidate scratch is a fixed 16 MiB array inside the library:
 * m * min(k, n) must not exceed 2,097,152 (SSG_EINVAL otherwise).  The array
 * is reserved on a device by the first call into this library there (the
 * module loads lazily), so a caller whose pool will take the whole GPU should
 * make one small call first.  Each uncaptured call looks up the array's
 * device address; a captured call reuses the one found by the last uncaptured
 * call on the device, so make the first call before any stream capture.
 * Buffers must be aligned to their element (8 bytes for sketches, 4 for the
 * rest; SSG_EINVAL otherwise).  The work is enqueued on `stream` (a
 * cudaStream_t, NULL = default stream) and the call returns without waiting
 * for it.  All calls share the array: calls that overlap on the GPU race,
 * calls ordered on one stream do not. */
int ssg_knn_noalloc(int metric, const void *dev_db, int64_t dim, int64_t n,
                    const void *dev_q, int64_t m, int32_t k,
                    uint32_t *dev_ids, float *dev_dists, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SSGPU_H */
