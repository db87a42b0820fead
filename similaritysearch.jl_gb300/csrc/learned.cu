// learned.cu -- the learned shortlist: training, embedding and search.
//
// A small network f: R^d -> R^E (d -> H (ReLU) -> E, or a fixed Gaussian
// random projection d -> E when H = 0) is trained so that exact neighbours are
// close in the embedding: triplets (anchor, one of its exact 10 nearest
// neighbours, a uniformly random object) are mined with this library's own
// exact allknn over a seeded sample of the database, and the triplet loss
// max(0, |f(a)-f(p)|^2 - |f(a)-f(n)|^2 + margin) is minimised with Adam on
// FP32 master weights (forward / backward kernels in mlp.cu).  After
// training every database row is embedded and indexed by a BF16 SqL2 index of
// dimension E (tensor-core scan).  A learned search embeds the queries, shortlists the
// S nearest embeddings, re-scores those S candidates with the exact FP32
// distance of the parent index and keeps the k best.  The recall of that
// pipeline against the plain method is estimated at training time on held-out
// objects; below the target (0.99 by default) searches fall back to the
// plain exhaustive method.
#include "ssgpu.h"
#include "common.cuh"
#include "kernels.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

namespace ssg {

struct LearnedModel {
    int64_t d = 0, H = 0, E = 0;
    float *W1 = nullptr, *b1 = nullptr, *W2 = nullptr, *b2 = nullptr;  // FP32 master weights
    ssg_index *sub = nullptr;                                            // plain SqL2 index over the embeddings
    int shortlist = 512;
    double est_recall = 0.0;
    double train_loss = 0.0;
    double train_seconds = 0.0;
    int64_t train_steps = 0;
    std::vector<float> loss_curve;
    // search scratch
    float *zq = nullptr, *hq = nullptr;
    uint32_t *cand_ids = nullptr;
    float *cand_d = nullptr;
    size_t zq_rows = 0, cand_rows = 0;
    int *dev_err = nullptr;  // status word of the tensor-core GEMMs' bounded waits
};

namespace {

struct Cuda {
    std::string err;
    bool ok(cudaError_t e, const char *what) {
        if (e == cudaSuccess) return true;
        err = std::string(what) + ": " + cudaGetErrorString(e);
        cudaGetLastError();
        return false;
    }
};

#define LK(call, what)                             \
    do {                                           \
        if (!cu.ok((call), (what))) return SSG_ECUDA; \
    } while (0)

void free_model_buffers(LearnedModel *m) {
    for (float *p : {m->W1, m->b1, m->W2, m->b2, m->zq, m->hq, m->cand_d}) if (p) cudaFree(p);
    if (m->cand_ids) cudaFree(m->cand_ids);
    if (m->dev_err) cudaFree(m->dev_err);
    m->W1 = m->b1 = m->W2 = m->b2 = m->zq = m->hq = m->cand_d = nullptr;
    m->cand_ids = nullptr;
    m->dev_err = nullptr;
    m->zq_rows = m->cand_rows = 0;
    if (m->sub) ssg_destroy(m->sub);
    m->sub = nullptr;
}

// Z (rows x E) = f(X) for rows of X (d floats); Hs is rows x H scratch.
// Tensor-core products with BF16 operands, as in training.
int embed_rows(LearnedModel *m, const float *X, int64_t rows, float *Z, float *Hs, int *err, cudaStream_t st, Cuda &cu,
               int *launches) {
    MlpGemm g;
    g.err = err;
    g.M = int(rows);
    if (m->H > 0) {
        g.A = X; g.lda = m->d; g.B = m->W1; g.ldb = m->d; g.C = Hs; g.ldc = m->H;
        g.N = int(m->H); g.K = int(m->d); g.bias = m->b1; g.relu = 1;
        LK(mlp_gemm(g, st, launches), "embedding");
        g.A = Hs; g.lda = m->H; g.B = m->W2; g.ldb = m->H; g.C = Z; g.ldc = m->E;
        g.N = int(m->E); g.K = int(m->H); g.bias = m->b2; g.relu = 0;
        LK(mlp_gemm(g, st, launches), "embedding");
    } else {
        g.A = X; g.lda = m->d; g.B = m->W1; g.ldb = m->d; g.C = Z; g.ldc = m->E;
        g.N = int(m->E); g.K = int(m->d);
        LK(mlp_gemm(g, st, launches), "embedding");
    }
    return SSG_OK;
}

// The model's device status word (zeroed); null after an allocation failure.
int *err_word(LearnedModel *m, Cuda &cu) {
    if (!m->dev_err) {
        void *p = nullptr;
        if (!cu.ok(cudaMalloc(&p, sizeof(int)), "allocating a status word")) return nullptr;
        m->dev_err = static_cast<int *>(p);
    }
    if (!cu.ok(cudaMemset(m->dev_err, 0, sizeof(int)), "clearing a status word")) return nullptr;
    return m->dev_err;
}

// After a synchronisation: SSG_ETIMEOUT if a bounded wait of the GEMMs gave up.
int check_err_word(LearnedModel *m, Cuda &cu) {
    int h = 0;
    if (!cu.ok(cudaMemcpy(&h, m->dev_err, sizeof(int), cudaMemcpyDeviceToHost), "reading a status word"))
        return SSG_ECUDA;
    if (h != 0) {
        cu.err = "a bounded wait in the network's tensor-core GEMM gave up (code " + std::to_string(h) + ")";
        return SSG_ETIMEOUT;
    }
    return SSG_OK;
}

float *dmalloc(size_t n, Cuda &cu, const char *what) {
    void *p = nullptr;
    if (!cu.ok(cudaMalloc(&p, n * 4), what)) return nullptr;
    return static_cast<float *>(p);
}

}  // namespace

void learned_free(LearnedModel *m) {
    if (!m) return;
    free_model_buffers(m);
    delete m;
}

double learned_get(const LearnedModel *m, const char *key, bool *found) {
    *found = true;
    if (!strcmp(key, "learned_recall")) return m ? m->est_recall : 0.0;
    if (!strcmp(key, "train_loss")) return m ? m->train_loss : 0.0;
    if (!strcmp(key, "train_seconds")) return m ? m->train_seconds : 0.0;
    if (!strcmp(key, "train_steps")) return m ? double(m->train_steps) : 0.0;
    if (!strcmp(key, "shortlist")) return m ? m->shortlist : 0.0;
    if (!strcmp(key, "learned_ready")) return m ? 1.0 : 0.0;
    *found = false;
    return 0.0;
}

bool learned_set(LearnedModel *m, const char *key, double v) {
    if (!strcmp(key, "shortlist") && m) {
        m->shortlist = int(v);
        return true;
    }
    return false;
}

// Embeds the whole database and (re)builds the shortlist index.
int learned_index_db(LearnedModel *m, const IndexView &v, std::string &err) {
    Cuda cu;
    const int64_t chunk = 65536;
    float *Z = dmalloc(size_t(v.n) * m->E, cu, "allocating embeddings");
    float *Hs = m->H > 0 ? dmalloc(size_t(chunk) * m->H, cu, "allocating hidden scratch") : nullptr;
    if (!Z || (m->H > 0 && !Hs)) { err = cu.err; if (Z) cudaFree(Z); return SSG_ENOMEM; }
    int rc = SSG_OK;
    int *ew = err_word(m, cu);
    if (!ew) rc = SSG_ECUDA;
    for (int64_t r0 = 0; r0 < v.n && rc == SSG_OK; r0 += chunk) {
        const int64_t rows = std::min(chunk, v.n - r0);
        rc = embed_rows(m, v.db + size_t(r0) * v.dim, rows, Z + size_t(r0) * m->E, Hs, ew, v.stream, cu, v.launches);
    }
    if (rc == SSG_OK && !cu.ok(cudaStreamSynchronize(v.stream), "embedding the database")) rc = SSG_ECUDA;
    if (rc == SSG_OK) rc = check_err_word(m, cu);
    if (rc == SSG_OK) {
        if (m->sub) ssg_destroy(m->sub);
        m->sub = nullptr;
        // BF16 tensor-core scan of the embeddings; long shortlists take its
        // threshold-filter path, the exact FP32 rerank in the parent's space
        // follows in learned_search
        rc = ssg_create_device(SSG_METRIC_SQL2, SSG_ELEM_F32, m->E, v.n, Z, m->E, SSG_PREC_BF16, &m->sub);
        if (!rc) rc = ssg_set_param(m->sub, "overfetch", 1.0);
        if (rc) {
            char buf[256];
            ssg_last_error(nullptr, buf, sizeof buf);
            cu.err = buf;
        }
    }
    cudaFree(Z);
    if (Hs) cudaFree(Hs);
    if (rc) err = cu.err;
    return rc;
}

// Learned search: embed, shortlist S in the embedding, exact rerank, top k.
int learned_search(LearnedModel *m, const IndexView &v, const float *dq, const float *dqn, int64_t mq, int k,
                   uint32_t *d_ids, float *d_dists, std::string &err) {
    Cuda cu;
    const int S = int(std::min<int64_t>(std::max(m->shortlist, k), v.n));
    if (size_t(mq) > m->zq_rows) {
        if (m->zq) cudaFree(m->zq);
        if (m->hq) cudaFree(m->hq);
        m->zq = dmalloc(size_t(mq) * m->E, cu, "allocating query embeddings");
        m->hq = m->H > 0 ? dmalloc(size_t(mq) * m->H, cu, "allocating query hidden layer") : nullptr;
        if (!m->zq || (m->H > 0 && !m->hq)) { err = cu.err; m->zq_rows = 0; return SSG_ENOMEM; }
        m->zq_rows = size_t(mq);
    }
    if (size_t(mq) * S > m->cand_rows) {
        if (m->cand_ids) cudaFree(m->cand_ids);
        if (m->cand_d) cudaFree(m->cand_d);
        void *p = nullptr;
        if (!cu.ok(cudaMalloc(&p, size_t(mq) * S * 4), "allocating candidates")) { err = cu.err; return SSG_ENOMEM; }
        m->cand_ids = static_cast<uint32_t *>(p);
        m->cand_d = dmalloc(size_t(mq) * S, cu, "allocating candidates");
        if (!m->cand_d) { err = cu.err; return SSG_ENOMEM; }
        m->cand_rows = size_t(mq) * S;
    }
    int *ew = err_word(m, cu);
    if (!ew) { err = cu.err; return SSG_ECUDA; }
    int rc = embed_rows(m, dq, mq, m->zq, m->hq, ew, v.stream, cu, v.launches);
    if (rc) { err = cu.err; return rc; }
    if (!cu.ok(cudaStreamSynchronize(v.stream), "embedding queries")) { err = cu.err; return SSG_ECUDA; }
    rc = check_err_word(m, cu);
    if (rc) { err = cu.err; return rc; }
    rc = ssg_search_device(m->sub, m->zq, mq, S, m->cand_ids, m->cand_d, 0);
    if (rc) {
        char buf[256];
        ssg_last_error(m->sub, buf, sizeof buf);
        err = std::string("shortlist search: ") + buf;
        return rc;
    }
    LK(launch_rerank(v.metric, v.db, v.db_norm, v.dim, dq, dqn, mq, S, m->cand_ids, m->cand_d, v.stream, v.launches),
       "re-ranking the shortlist");
    LK(cudaMemcpy2DAsync(d_ids, size_t(k) * 4, m->cand_ids, size_t(S) * 4, size_t(k) * 4, size_t(mq),
                         cudaMemcpyDeviceToDevice, v.stream),
       "copying ids");
    LK(cudaMemcpy2DAsync(d_dists, size_t(k) * 4, m->cand_d, size_t(S) * 4, size_t(k) * 4, size_t(mq),
                         cudaMemcpyDeviceToDevice, v.stream),
       "copying distances");
    if (!cu.ok(cudaStreamSynchronize(v.stream), "learned search")) { err = cu.err; return SSG_ECUDA; }
    (void)cu;
    return SSG_OK;
}

// Trains a model on the index's database (see the file comment).
int learned_train(const IndexView &v, const TrainArgs &t, LearnedModel **out, std::string &err) {
    Cuda cu;
    const auto t0 = std::chrono::steady_clock::now();
    std::mt19937_64 rng(t.seed);
    const int64_t ns = std::min<int64_t>(t.sample, v.n);
    if (ns < 12) { err = "the training sample needs at least 12 objects"; return SSG_EINVAL; }
    LearnedModel *m = new LearnedModel();
    m->d = v.dim;
    m->H = t.hidden;
    m->E = t.out_dim;
    m->shortlist = t.shortlist;
    const int64_t d = v.dim, H = t.hidden, E = t.out_dim;
    auto fail = [&](int code) {
        err = cu.err.empty() ? err : cu.err;
        learned_free(m);
        return code;
    };
    // weights (He initialisation; a random projection when H == 0)
    std::normal_distribution<float> nd(0.0f, 1.0f);
    std::vector<float> w1(size_t(H > 0 ? H : E) * d), w2(size_t(E) * (H > 0 ? H : 1));
    const float s1 = H > 0 ? std::sqrt(2.0f / float(d)) : 1.0f / std::sqrt(float(d));
    for (auto &x : w1) x = nd(rng) * s1;
    const float s2 = H > 0 ? std::sqrt(1.0f / float(H)) : 0.0f;
    for (auto &x : w2) x = nd(rng) * s2;
    m->W1 = dmalloc(w1.size(), cu, "allocating weights");
    if (!m->W1 || !cu.ok(cudaMemcpy(m->W1, w1.data(), w1.size() * 4, cudaMemcpyHostToDevice), "uploading weights"))
        return fail(SSG_ECUDA);
    if (H > 0) {
        m->b1 = dmalloc(size_t(H), cu, "allocating weights");
        m->W2 = dmalloc(w2.size(), cu, "allocating weights");
        m->b2 = dmalloc(size_t(E), cu, "allocating weights");
        if (!m->b1 || !m->W2 || !m->b2) return fail(SSG_ENOMEM);
        if (!cu.ok(cudaMemset(m->b1, 0, size_t(H) * 4), "init") || !cu.ok(cudaMemset(m->b2, 0, size_t(E) * 4), "init") ||
            !cu.ok(cudaMemcpy(m->W2, w2.data(), w2.size() * 4, cudaMemcpyHostToDevice), "uploading weights"))
            return fail(SSG_ECUDA);
    }
    if (H > 0 && t.epochs > 0 && t.triplets > 0) {
        // 1. seeded sample of the database
        std::vector<int64_t> perm(size_t(v.n));
        for (int64_t i = 0; i < v.n; ++i) perm[size_t(i)] = i;
        for (int64_t i = 0; i < ns; ++i) {
            std::uniform_int_distribution<int64_t> u(i, v.n - 1);
            std::swap(perm[size_t(i)], perm[size_t(u(rng))]);
        }
        int64_t *d_sample = nullptr;
        float *S = nullptr;
        LK(cudaMalloc(&d_sample, size_t(ns) * 8), "allocating the sample");
        S = dmalloc(size_t(ns) * d, cu, "allocating the sample");
        if (!S) { cudaFree(d_sample); return fail(SSG_ENOMEM); }
        cudaMemcpy(d_sample, perm.data(), size_t(ns) * 8, cudaMemcpyHostToDevice);
        LK(launch_gather_rows(v.db, d_sample, ns, size_t(d) * 4, S, v.stream, v.launches), "gathering the sample");
        LK(cudaStreamSynchronize(v.stream), "gathering the sample");
        cudaFree(d_sample);
        // 2. exact nearest neighbours of every sampled object (self excluded)
        // with this library: 10 positives, and 40 more ranks for the
        // semi-hard negatives when t.hard > 0
        const int KP = int(std::min<int64_t>(10, ns - 1));
        const int KN = t.hard > 0.0f ? int(std::min<int64_t>(40, ns - 1 - KP)) : 0;
        const int KA = KP + KN;
        ssg_index *tmp = nullptr;
        int rc = ssg_create_device(v.metric, SSG_ELEM_F32, d, ns, S, d, SSG_PREC_FP32, &tmp);
        if (rc) { cudaFree(S); err = "sample index creation failed"; learned_free(m); return rc; }
        uint32_t *nn_ids = nullptr;
        float *nn_d = nullptr;
        if (cudaMalloc(&nn_ids, size_t(ns) * KA * 4) != cudaSuccess || cudaMalloc(&nn_d, size_t(ns) * KA * 4) != cudaSuccess) {
            cudaGetLastError();
            if (nn_ids) cudaFree(nn_ids);
            ssg_destroy(tmp);
            cudaFree(S);
            err = "allocating the sample's neighbours";
            learned_free(m);
            return SSG_ENOMEM;
        }
        rc = ssg_allknn_device(tmp, KA, 1, nn_ids, nn_d);
        std::vector<uint32_t> nn(size_t(ns) * KA);
        if (!rc) cudaMemcpy(nn.data(), nn_ids, nn.size() * 4, cudaMemcpyDeviceToHost);
        ssg_destroy(tmp);
        cudaFree(nn_ids);
        cudaFree(nn_d);
        if (rc) { cudaFree(S); err = "allknn over the sample failed"; learned_free(m); return rc; }
        // 3. triplets (indices into the sample): anchor, one of its KP exact
        // neighbours, and a negative -- with probability t.hard one of its
        // neighbours ranked KP+1 .. KP+KN (close but farther than every
        // positive: the anchor's neighbourhood must be ordered, not only
        // separated from far objects), otherwise a uniform object
        const int64_t T = t.triplets;
        std::vector<int64_t> trip(size_t(3 * T));
        std::uniform_int_distribution<int64_t> ua(0, ns - 1);
        std::uniform_int_distribution<int> ur(0, KP - 1);
        std::uniform_int_distribution<int> uh(0, std::max(0, KN - 1));
        std::uniform_real_distribution<float> u01(0.0f, 1.0f);
        for (int64_t i = 0; i < T; ++i) {
            const int64_t a = ua(rng);
            uint32_t p = nn[size_t(a) * KA + size_t(ur(rng))];
            if (p == 0) p = uint32_t(a + 1);  // unfilled slot: the anchor itself
            int64_t neg = -1;
            if (KN > 0 && u01(rng) < t.hard) {
                const uint32_t h = nn[size_t(a) * KA + KP + size_t(uh(rng))];
                if (h != 0) neg = int64_t(h) - 1;
            }
            if (neg < 0) neg = ua(rng);
            trip[size_t(i)] = a;
            trip[size_t(T + i)] = int64_t(p) - 1;
            trip[size_t(2 * T + i)] = neg;
        }
        int64_t *d_trip = nullptr;
        LK(cudaMalloc(&d_trip, trip.size() * 8), "allocating triplets");
        cudaMemcpy(d_trip, trip.data(), trip.size() * 8, cudaMemcpyHostToDevice);
        // 4. training buffers.  One step: X = the batch's anchors, positives
        // and negatives (3B rows), H = relu(X W1^T + b1), Z = H W2^T + b2,
        // the loss and dZ, gW2 = dZ^T H, dH = (dZ W2) * (H > 0) with its
        // per-tile column sums (gb1), gW1 = dH^T X, the column sums of dZ
        // (gb2), then Adam summing each gradient's parts in a fixed order.
        // Every product runs on the tensor cores (mlp.cu) split along K so
        // that each CTA walks about two K-blocks (the products are small:
        // one CTA per output tile would serialise a global-load round trip
        // per K-block); the forward products' parts are summed by a reduction
        // that applies the bias and the ReLU.
        const int B = t.batch;
        const int R = 3 * B;
        const int mt = mlp_gemm_mtiles(R);                 // row tiles: parts of gb1
        const int kWant = 2 * device_sm_count();           // CTAs per product
        const int sf1 = mlp_splits(int(d), mt * mlp_gemm_ntiles(int(H)), kWant);
        const int sf2 = mlp_splits(int(H), mt * mlp_gemm_ntiles(int(E)), kWant);
        const int s1 = mlp_splits(R, mlp_gemm_mtiles(int(H)) * mlp_gemm_ntiles(int(d)), kWant);
        const int s2 = mlp_splits(R, mlp_gemm_mtiles(int(E)) * mlp_gemm_ntiles(int(H)), kWant);
        const int pb2 = std::max(1, std::min(32, R / 96)); // row ranges of gb2's column sums
        float *X = dmalloc(size_t(R) * d, cu, "x"), *Hh = dmalloc(size_t(R) * H, cu, "h"), *Z = dmalloc(size_t(R) * E, cu, "z");
        float *dZ = dmalloc(size_t(R) * E, cu, "dz"), *dH = dmalloc(size_t(R) * H, cu, "dh");
        float *P = dmalloc(std::max(size_t(sf1) * R * H, size_t(sf2) * R * E), cu, "parts");
        float *gW1 = dmalloc(size_t(s1) * H * d, cu, "g"), *gb1 = dmalloc(size_t(mt) * H, cu, "g");
        float *gW2 = dmalloc(size_t(s2) * E * H, cu, "g"), *gb2 = dmalloc(size_t(pb2) * E, cu, "g");
        const size_t npar = size_t(H) * d + H + size_t(E) * H + E;
        float *mom = dmalloc(2 * npar, cu, "adam");
        float *stat = dmalloc(2, cu, "loss");
        int *ew = err_word(m, cu);
        if (!X || !Hh || !Z || !dZ || !dH || !P || !gW1 || !gb1 || !gW2 || !gb2 || !mom || !stat || !ew) {
            for (float *p : {X, Hh, Z, dZ, dH, P, gW1, gb1, gW2, gb2, mom, stat})
                if (p) cudaFree(p);
            cudaFree(S); cudaFree(d_trip);
            return fail(SSG_ENOMEM);
        }
        cudaMemset(mom, 0, 2 * npar * 4);
        float *mW1 = mom, *mb1 = mW1 + size_t(H) * d, *mW2 = mb1 + H, *mb2 = mW2 + size_t(E) * H;
        float *vW1 = mom + npar, *vb1 = vW1 + size_t(H) * d, *vW2 = vb1 + H, *vb2 = vW2 + size_t(E) * H;
        const int64_t steps_per_epoch = (T + B - 1) / B;
        int64_t step = 0;
        int status = SSG_OK;
        for (int ep = 0; ep < t.epochs && status == SSG_OK; ++ep) {
            for (int64_t s = 0; s < steps_per_epoch && status == SSG_OK; ++s) {
                const int64_t off = (s * B) % T;
                const int bb = int(std::min<int64_t>(B, T - off));
                const int rows = 3 * bb;
                ++step;
                MlpGemm f1, f2, gw2, dh, gw1;
                f1.err = f2.err = gw2.err = dh.err = gw1.err = ew;
                // parts of X W1^T, then H = relu(sum + b1)
                f1.A = X; f1.lda = d; f1.B = m->W1; f1.ldb = d; f1.C = P; f1.ldc = H;
                f1.M = rows; f1.N = int(H); f1.K = int(d); f1.splits = sf1;
                // parts of H W2^T, then Z = sum + b2
                f2.A = Hh; f2.lda = H; f2.B = m->W2; f2.ldb = H; f2.C = P; f2.ldc = E;
                f2.M = rows; f2.N = int(E); f2.K = int(H); f2.splits = sf2;
                // gW2 (E x H) = dZ^T H: both operands transposed, K = rows
                gw2.A = dZ; gw2.lda = E; gw2.a_kmajor = 0; gw2.B = Hh; gw2.ldb = H; gw2.b_kmajor = 0;
                gw2.C = gW2; gw2.ldc = H; gw2.M = int(E); gw2.N = int(H); gw2.K = rows; gw2.splits = s2;
                // dH = (dZ W2) * (H > 0), column sums per row tile (gb1); K = E
                dh.A = dZ; dh.lda = E; dh.B = m->W2; dh.ldb = H; dh.b_kmajor = 0; dh.C = dH; dh.ldc = H;
                dh.M = rows; dh.N = int(H); dh.K = int(E); dh.mask = Hh; dh.colsum = gb1;
                // gW1 (H x d) = dH^T X, K = rows
                gw1.A = dH; gw1.lda = H; gw1.a_kmajor = 0; gw1.B = X; gw1.ldb = d; gw1.b_kmajor = 0;
                gw1.C = gW1; gw1.ldc = d; gw1.M = int(H); gw1.N = int(d); gw1.K = rows; gw1.splits = s1;
                const int mt_b = mlp_gemm_mtiles(rows);
                float *const aw[4] = {m->W1, m->b1, m->W2, m->b2};
                const float *const ag[4] = {gW1, gb1, gW2, gb2};
                const int ap[4] = {s1, mt_b, s2, pb2};
                float *const am[4] = {mW1, mb1, mW2, mb2};
                float *const av[4] = {vW1, vb1, vW2, vb2};
                const int64_t ac[4] = {int64_t(H) * d, H, int64_t(E) * H, E};
                bool ok = cu.ok(mlp_gather3(S, d_trip, T, off, bb, int(d), X, v.stream, v.launches), "gathering a batch") &&
                          cu.ok(cudaMemsetAsync(stat, 0, 8, v.stream), "loss") &&
                          cu.ok(mlp_gemm(f1, v.stream, v.launches), "fwd") &&
                          cu.ok(mlp_reduce_parts(P, sf1, rows, int(H), m->b1, 1, Hh, v.stream, v.launches), "fwd") &&
                          cu.ok(mlp_gemm(f2, v.stream, v.launches), "fwd") &&
                          cu.ok(mlp_reduce_parts(P, sf2, rows, int(E), m->b2, 0, Z, v.stream, v.launches), "fwd") &&
                          cu.ok(mlp_triplet(Z, bb, int(E), t.margin, dZ, stat, reinterpret_cast<int *>(stat + 1),
                                            v.stream, v.launches), "loss") &&
                          cu.ok(mlp_gemm(gw2, v.stream, v.launches), "bwd") &&
                          cu.ok(mlp_colsum_parts(dZ, rows, int(E), pb2, gb2, v.stream, v.launches), "bwd") &&
                          cu.ok(mlp_gemm(dh, v.stream, v.launches), "bwd") &&
                          cu.ok(mlp_gemm(gw1, v.stream, v.launches), "bwd") &&
                          cu.ok(mlp_adam4(aw, ag, ap, am, av, ac, t.lr, int(step), v.stream, v.launches), "adam");
                if (!ok) status = SSG_ECUDA;
                if (ok && (s + 1 == steps_per_epoch)) {
                    float loss = 0.0f;
                    cudaMemcpyAsync(&loss, stat, 4, cudaMemcpyDeviceToHost, v.stream);
                    if (!cu.ok(cudaStreamSynchronize(v.stream), "training")) status = SSG_ECUDA;
                    if (status == SSG_OK) status = check_err_word(m, cu);
                    m->loss_curve.push_back(loss);
                    m->train_loss = loss;
                }
            }
        }
        m->train_steps = step;
        for (float *p : {X, Hh, Z, dZ, dH, P, gW1, gb1, gW2, gb2, mom, stat, S}) cudaFree(p);
        cudaFree(d_trip);
        if (status) return fail(status);
    }
    int rc = learned_index_db(m, v, err);
    if (rc) { learned_free(m); return rc; }
    m->train_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *out = m;
    return SSG_OK;
}

// -- model files: "SSGMLP01", int64 d, H, E, then W1, b1, W2, b2 (little-endian f32)
int learned_save(const LearnedModel *m, const char *path, std::string &err) {
    FILE *f = fopen(path, "wb");
    if (!f) { err = "cannot open the model file for writing"; return SSG_EINVAL; }
    const char magic[8] = {'S', 'S', 'G', 'M', 'L', 'P', '0', '1'};
    int64_t hdr[3] = {m->d, m->H, m->E};
    fwrite(magic, 1, 8, f);
    fwrite(hdr, 8, 3, f);
    auto put = [&](const float *dev, size_t n) {
        std::vector<float> h(n);
        if (n) cudaMemcpy(h.data(), dev, n * 4, cudaMemcpyDeviceToHost);
        fwrite(h.data(), 4, n, f);
    };
    if (m->H > 0) {
        put(m->W1, size_t(m->H) * m->d);
        put(m->b1, size_t(m->H));
        put(m->W2, size_t(m->E) * m->H);
        put(m->b2, size_t(m->E));
    } else {
        put(m->W1, size_t(m->E) * m->d);
    }
    const bool ok = fclose(f) == 0;
    if (!ok) { err = "writing the model file failed"; return SSG_EINVAL; }
    return SSG_OK;
}

int learned_load(const IndexView &v, const char *path, LearnedModel **out, std::string &err) {
    FILE *f = fopen(path, "rb");
    if (!f) { err = "cannot open the model file"; return SSG_EINVAL; }
    char magic[8];
    int64_t hdr[3];
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, "SSGMLP01", 8) != 0 || fread(hdr, 8, 3, f) != 3) {
        fclose(f);
        err = "not a model file";
        return SSG_EINVAL;
    }
    if (hdr[0] != v.dim || hdr[1] < 0 || hdr[2] <= 0 || hdr[1] > 8192 || hdr[2] > 256) {
        fclose(f);
        err = "the model's input dimension does not match the index";
        return SSG_EINVAL;
    }
    LearnedModel *m = new LearnedModel();
    m->d = hdr[0];
    m->H = hdr[1];
    m->E = hdr[2];
    Cuda cu;
    auto get = [&](float **dev, size_t n) -> bool {
        std::vector<float> h(n);
        if (fread(h.data(), 4, n, f) != n) return false;
        *dev = dmalloc(n, cu, "allocating weights");
        return *dev && cudaMemcpy(*dev, h.data(), n * 4, cudaMemcpyHostToDevice) == cudaSuccess;
    };
    bool ok = m->H > 0 ? (get(&m->W1, size_t(m->H) * m->d) && get(&m->b1, size_t(m->H)) &&
                          get(&m->W2, size_t(m->E) * m->H) && get(&m->b2, size_t(m->E)))
                       : get(&m->W1, size_t(m->E) * m->d);
    fclose(f);
    if (!ok) { err = "truncated model file"; learned_free(m); return SSG_EINVAL; }
    int rc = learned_index_db(m, v, err);
    if (rc) { learned_free(m); return rc; }
    *out = m;
    return SSG_OK;
}

void learned_set_recall(LearnedModel *m, double r) { m->est_recall = r; }

// One forward + backward pass on a host batch (anchors; positives; negatives)
// with host weights: the gradient check against the CPU oracle.  The same
// kernels and decomposition as a training step (split K, per-tile column
// sums, parts summed in order), with the GEMMs in exact mode (operands as
// three BF16 pieces, six piece products), so the result is checked at
// FP32-class accuracy.
int learned_grad_check(int64_t d, int64_t H, int64_t E, const float *W1, const float *b1, const float *W2,
                       const float *b2, const float *X, int B, float margin, float *loss, float *gW1, float *gb1,
                       float *gW2, float *gb2, std::string &err) {
    Cuda cu;
    const int R = 3 * B;
    const int mt = mlp_gemm_mtiles(R);
    const int kWant = 2 * device_sm_count();
    const int sf1 = mlp_splits(int(d), mt * mlp_gemm_ntiles(int(H)), kWant);
    const int sf2 = mlp_splits(int(H), mt * mlp_gemm_ntiles(int(E)), kWant);
    const int s1 = mlp_splits(R, mlp_gemm_mtiles(int(H)) * mlp_gemm_ntiles(int(d)), kWant);
    const int s2 = mlp_splits(R, mlp_gemm_mtiles(int(E)) * mlp_gemm_ntiles(int(H)), kWant);
    const int pb2 = std::max(1, std::min(32, R / 96));
    std::vector<void *> bufs;
    auto up = [&](const float *h, size_t n) -> float * {
        float *p = dmalloc(n, cu, "alloc");
        if (p) { bufs.push_back(p); cudaMemcpy(p, h, n * 4, cudaMemcpyHostToDevice); }
        return p;
    };
    auto mk = [&](size_t n) -> float * {
        float *p = dmalloc(n, cu, "alloc");
        if (p) bufs.push_back(p);
        return p;
    };
    float *dW1 = up(W1, size_t(H) * d), *db1 = up(b1, H), *dW2 = up(W2, size_t(E) * H), *db2 = up(b2, E);
    float *dX = up(X, size_t(R) * d), *Hh = mk(size_t(R) * H), *Z = mk(size_t(R) * E), *dZ = mk(size_t(R) * E);
    float *dH = mk(size_t(R) * H), *p1 = mk(size_t(s1) * H * d), *pb1 = mk(size_t(mt) * H), *p2 = mk(size_t(s2) * E * H);
    float *pf = mk(std::max(size_t(sf1) * R * H, size_t(sf2) * R * E));
    float *pb2d = mk(size_t(pb2) * E), *g1 = mk(size_t(H) * d), *gb1d = mk(H), *g2 = mk(size_t(E) * H);
    float *gb2d = mk(E), *stat = mk(2);
    int *ew = reinterpret_cast<int *>(mk(1));
    int rc = SSG_OK;
    for (void *p : {(void *)dW1, (void *)db1, (void *)dW2, (void *)db2, (void *)dX, (void *)Hh, (void *)Z, (void *)dZ,
                    (void *)dH, (void *)p1, (void *)pb1, (void *)p2, (void *)pf, (void *)pb2d, (void *)g1, (void *)gb1d,
                    (void *)g2, (void *)gb2d, (void *)stat, (void *)ew})
        if (!p) rc = SSG_ENOMEM;
    cudaStream_t st = nullptr;
    if (!rc) {
        cudaMemset(stat, 0, 8);
        cudaMemset(ew, 0, 4);
        MlpGemm f1, f2, gw2, dh, gw1;
        f1.err = f2.err = gw2.err = dh.err = gw1.err = ew;
        f1.exact = f2.exact = gw2.exact = dh.exact = gw1.exact = 1;
        f1.A = dX; f1.lda = d; f1.B = dW1; f1.ldb = d; f1.C = pf; f1.ldc = H;
        f1.M = R; f1.N = int(H); f1.K = int(d); f1.splits = sf1;
        f2.A = Hh; f2.lda = H; f2.B = dW2; f2.ldb = H; f2.C = pf; f2.ldc = E;
        f2.M = R; f2.N = int(E); f2.K = int(H); f2.splits = sf2;
        gw2.A = dZ; gw2.lda = E; gw2.a_kmajor = 0; gw2.B = Hh; gw2.ldb = H; gw2.b_kmajor = 0;
        gw2.C = p2; gw2.ldc = H; gw2.M = int(E); gw2.N = int(H); gw2.K = R; gw2.splits = s2;
        dh.A = dZ; dh.lda = E; dh.B = dW2; dh.ldb = H; dh.b_kmajor = 0; dh.C = dH; dh.ldc = H;
        dh.M = R; dh.N = int(H); dh.K = int(E); dh.mask = Hh; dh.colsum = pb1;
        gw1.A = dH; gw1.lda = H; gw1.a_kmajor = 0; gw1.B = dX; gw1.ldb = d; gw1.b_kmajor = 0;
        gw1.C = p1; gw1.ldc = d; gw1.M = int(H); gw1.N = int(d); gw1.K = R; gw1.splits = s1;
        bool ok = cu.ok(mlp_gemm(f1, st, nullptr), "fwd") &&
                  cu.ok(mlp_reduce_parts(pf, sf1, R, int(H), db1, 1, Hh, st, nullptr), "fwd") &&
                  cu.ok(mlp_gemm(f2, st, nullptr), "fwd") &&
                  cu.ok(mlp_reduce_parts(pf, sf2, R, int(E), db2, 0, Z, st, nullptr), "fwd") &&
                  cu.ok(mlp_triplet(Z, B, int(E), margin, dZ, stat, reinterpret_cast<int *>(stat + 1), st, nullptr), "loss") &&
                  cu.ok(mlp_gemm(gw2, st, nullptr), "bwd") &&
                  cu.ok(mlp_colsum_parts(dZ, R, int(E), pb2, pb2d, st, nullptr), "bwd") &&
                  cu.ok(mlp_gemm(dh, st, nullptr), "bwd") && cu.ok(mlp_gemm(gw1, st, nullptr), "bwd") &&
                  cu.ok(mlp_sum_parts(p1, s1, int64_t(H) * d, g1, st, nullptr), "sum") &&
                  cu.ok(mlp_sum_parts(pb1, mt, H, gb1d, st, nullptr), "sum") &&
                  cu.ok(mlp_sum_parts(p2, s2, int64_t(E) * H, g2, st, nullptr), "sum") &&
                  cu.ok(mlp_sum_parts(pb2d, pb2, E, gb2d, st, nullptr), "sum") && cu.ok(cudaDeviceSynchronize(), "sync");
        if (!ok) rc = SSG_ECUDA;
        int h = 0;
        if (!rc && cu.ok(cudaMemcpy(&h, ew, 4, cudaMemcpyDeviceToHost), "status") && h != 0) {
            cu.err = "a bounded wait in the network's tensor-core GEMM gave up";
            rc = SSG_ETIMEOUT;
        }
        if (!rc) {
            cudaMemcpy(loss, stat, 4, cudaMemcpyDeviceToHost);
            cudaMemcpy(gW1, g1, size_t(H) * d * 4, cudaMemcpyDeviceToHost);
            cudaMemcpy(gb1, gb1d, size_t(H) * 4, cudaMemcpyDeviceToHost);
            cudaMemcpy(gW2, g2, size_t(E) * H * 4, cudaMemcpyDeviceToHost);
            cudaMemcpy(gb2, gb2d, size_t(E) * 4, cudaMemcpyDeviceToHost);
        }
    }
    for (void *p : bufs) cudaFree(p);
    if (rc) err = cu.err;
    return rc;
}

}  // namespace ssg
