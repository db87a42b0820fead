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
    m->W1 = m->b1 = m->W2 = m->b2 = m->zq = m->hq = m->cand_d = nullptr;
    m->cand_ids = nullptr;
    m->zq_rows = m->cand_rows = 0;
    if (m->sub) ssg_destroy(m->sub);
    m->sub = nullptr;
}

// Z (rows x E) = f(X) for rows of X (d floats); Hs is rows x H scratch.
int embed_rows(LearnedModel *m, const float *X, int64_t rows, float *Z, float *Hs, cudaStream_t st, Cuda &cu,
               int *launches) {
    if (m->H > 0) {
        LK(mlp_gemm(X, m->W1, m->b1, Hs, int(rows), int(m->H), int(m->d), 0, 0, 1, 1, 0, st, launches), "embedding");
        LK(mlp_gemm(Hs, m->W2, m->b2, Z, int(rows), int(m->E), int(m->H), 0, 0, 0, 1, 0, st, launches), "embedding");
    } else {
        LK(mlp_gemm(X, m->W1, nullptr, Z, int(rows), int(m->E), int(m->d), 0, 0, 0, 1, 0, st, launches), "embedding");
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
    for (int64_t r0 = 0; r0 < v.n && rc == SSG_OK; r0 += chunk) {
        const int64_t rows = std::min(chunk, v.n - r0);
        rc = embed_rows(m, v.db + size_t(r0) * v.dim, rows, Z + size_t(r0) * m->E, Hs, v.stream, cu, v.launches);
    }
    if (rc == SSG_OK && !cu.ok(cudaStreamSynchronize(v.stream), "embedding the database")) rc = SSG_ECUDA;
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
    int rc = embed_rows(m, dq, mq, m->zq, m->hq, v.stream, cu, v.launches);
    if (rc) { err = cu.err; return rc; }
    if (!cu.ok(cudaStreamSynchronize(v.stream), "embedding queries")) { err = cu.err; return SSG_ECUDA; }
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
        // 2. exact 10-NN of every sampled object (self excluded) with this library
        ssg_index *tmp = nullptr;
        int rc = ssg_create_device(v.metric, SSG_ELEM_F32, d, ns, S, d, SSG_PREC_FP32, &tmp);
        if (rc) { cudaFree(S); err = "sample index creation failed"; learned_free(m); return rc; }
        uint32_t *nn_ids = nullptr;
        float *nn_d = nullptr;
        if (cudaMalloc(&nn_ids, size_t(ns) * 10 * 4) != cudaSuccess || cudaMalloc(&nn_d, size_t(ns) * 10 * 4) != cudaSuccess) {
            cudaGetLastError();
            if (nn_ids) cudaFree(nn_ids);
            ssg_destroy(tmp);
            cudaFree(S);
            err = "allocating the sample's neighbours";
            learned_free(m);
            return SSG_ENOMEM;
        }
        rc = ssg_allknn_device(tmp, 10, 1, nn_ids, nn_d);
        std::vector<uint32_t> nn(size_t(ns) * 10);
        if (!rc) cudaMemcpy(nn.data(), nn_ids, nn.size() * 4, cudaMemcpyDeviceToHost);
        ssg_destroy(tmp);
        cudaFree(nn_ids);
        cudaFree(nn_d);
        if (rc) { cudaFree(S); err = "allknn over the sample failed"; learned_free(m); return rc; }
        // 3. triplets (indices into the sample)
        const int64_t T = t.triplets;
        std::vector<int64_t> trip(size_t(3 * T));
        std::uniform_int_distribution<int64_t> ua(0, ns - 1);
        std::uniform_int_distribution<int> ur(0, 9);
        for (int64_t i = 0; i < T; ++i) {
            const int64_t a = ua(rng);
            uint32_t p = nn[size_t(a) * 10 + size_t(ur(rng))];
            if (p == 0) p = uint32_t(a + 1);  // unfilled slot: the anchor itself
            trip[size_t(i)] = a;
            trip[size_t(T + i)] = int64_t(p) - 1;
            trip[size_t(2 * T + i)] = ua(rng);
        }
        int64_t *d_trip = nullptr;
        LK(cudaMalloc(&d_trip, trip.size() * 8), "allocating triplets");
        cudaMemcpy(d_trip, trip.data(), trip.size() * 8, cudaMemcpyHostToDevice);
        // 4. training buffers
        const int B = t.batch;
        const size_t R = size_t(3) * B;
        float *X = dmalloc(R * d, cu, "x"), *Hh = dmalloc(R * H, cu, "h"), *Z = dmalloc(R * E, cu, "z");
        float *dZ = dmalloc(R * E, cu, "dz"), *dH = dmalloc(R * H, cu, "dh");
        float *gW1 = dmalloc(size_t(H) * d, cu, "g"), *gb1 = dmalloc(size_t(H), cu, "g");
        float *gW2 = dmalloc(size_t(E) * H, cu, "g"), *gb2 = dmalloc(size_t(E), cu, "g");
        const size_t npar = size_t(H) * d + H + size_t(E) * H + E;
        float *mom = dmalloc(2 * npar, cu, "adam");
        float *stat = dmalloc(2, cu, "loss");
        if (!X || !Hh || !Z || !dZ || !dH || !gW1 || !gb1 || !gW2 || !gb2 || !mom || !stat) {
            for (float *p : {X, Hh, Z, dZ, dH, gW1, gb1, gW2, gb2, mom, stat})
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
                const int64_t bb = std::min<int64_t>(B, T - off);
                // X = [anchors; positives; negatives] of this batch
                for (int part = 0; part < 3; ++part)
                    if (!cu.ok(launch_gather_rows(S, d_trip + part * T + off, bb, size_t(d) * 4,
                                                  X + size_t(part) * bb * d, v.stream, v.launches),
                               "gathering a batch")) status = SSG_ECUDA;
                const int rows = int(3 * bb);
                ++step;
                cudaMemsetAsync(stat, 0, 8, v.stream);
                bool ok = cu.ok(mlp_gemm(X, m->W1, m->b1, Hh, rows, int(H), int(d), 0, 0, 1, 1, 0, v.stream, v.launches), "fwd") &&
                          cu.ok(mlp_gemm(Hh, m->W2, m->b2, Z, rows, int(E), int(H), 0, 0, 0, 1, 0, v.stream, v.launches), "fwd") &&
                          cu.ok(mlp_triplet(Z, int(bb), int(E), t.margin, dZ, stat, reinterpret_cast<int *>(stat + 1),
                                            v.stream, v.launches), "loss") &&
                          cu.ok(mlp_gemm(dZ, Hh, nullptr, gW2, int(E), int(H), rows, 1, 1, 0, 1, 0, v.stream, v.launches), "bwd") &&
                          cu.ok(mlp_colsum(dZ, rows, int(E), gb2, v.stream, v.launches), "bwd") &&
                          cu.ok(mlp_gemm(dZ, m->W2, nullptr, dH, rows, int(H), int(E), 0, 1, 0, 1, 0, v.stream, v.launches), "bwd") &&
                          cu.ok(mlp_relu_backward(dH, Hh, int64_t(rows) * H, v.stream, v.launches), "bwd") &&
                          cu.ok(mlp_gemm(dH, X, nullptr, gW1, int(H), int(d), rows, 1, 1, 0, 1, 0, v.stream, v.launches), "bwd") &&
                          cu.ok(mlp_colsum(dH, rows, int(H), gb1, v.stream, v.launches), "bwd") &&
                          cu.ok(mlp_adam(m->W1, gW1, mW1, vW1, int64_t(H) * d, t.lr, int(step), v.stream, v.launches), "adam") &&
                          cu.ok(mlp_adam(m->b1, gb1, mb1, vb1, H, t.lr, int(step), v.stream, v.launches), "adam") &&
                          cu.ok(mlp_adam(m->W2, gW2, mW2, vW2, int64_t(E) * H, t.lr, int(step), v.stream, v.launches), "adam") &&
                          cu.ok(mlp_adam(m->b2, gb2, mb2, vb2, E, t.lr, int(step), v.stream, v.launches), "adam");
                if (!ok) status = SSG_ECUDA;
                if (ok && (s + 1 == steps_per_epoch)) {
                    float loss = 0.0f;
                    cudaMemcpyAsync(&loss, stat, 4, cudaMemcpyDeviceToHost, v.stream);
                    if (!cu.ok(cudaStreamSynchronize(v.stream), "training")) status = SSG_ECUDA;
                    m->loss_curve.push_back(loss);
                    m->train_loss = loss;
                }
            }
        }
        m->train_steps = step;
        for (float *p : {X, Hh, Z, dZ, dH, gW1, gb1, gW2, gb2, mom, stat, S}) cudaFree(p);
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
// with host weights: the gradient check against the CPU oracle.
int learned_grad_check(int64_t d, int64_t H, int64_t E, const float *W1, const float *b1, const float *W2,
                       const float *b2, const float *X, int B, float margin, float *loss, float *gW1, float *gb1,
                       float *gW2, float *gb2, std::string &err) {
    Cuda cu;
    const size_t R = size_t(3) * B;
    std::vector<float *> bufs;
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
    float *dX = up(X, R * d), *Hh = mk(R * H), *Z = mk(R * E), *dZ = mk(R * E), *dH = mk(R * H);
    float *g1 = mk(size_t(H) * d), *gb1d = mk(H), *g2 = mk(size_t(E) * H), *gb2d = mk(E), *stat = mk(2);
    int rc = SSG_OK;
    if (!dW1 || !db1 || !dW2 || !db2 || !dX || !Hh || !Z || !dZ || !dH || !g1 || !gb1d || !g2 || !gb2d || !stat)
        rc = SSG_ENOMEM;
    cudaStream_t st = nullptr;
    const int rows = int(R);
    if (!rc) {
        cudaMemset(stat, 0, 8);
        bool ok = cu.ok(mlp_gemm(dX, dW1, db1, Hh, rows, int(H), int(d), 0, 0, 1, 0, 0, st, nullptr), "fwd") &&
                  cu.ok(mlp_gemm(Hh, dW2, db2, Z, rows, int(E), int(H), 0, 0, 0, 0, 0, st, nullptr), "fwd") &&
                  cu.ok(mlp_triplet(Z, B, int(E), margin, dZ, stat, reinterpret_cast<int *>(stat + 1), st, nullptr), "loss") &&
                  cu.ok(mlp_gemm(dZ, Hh, nullptr, g2, int(E), int(H), rows, 1, 1, 0, 0, 0, st, nullptr), "bwd") &&
                  cu.ok(mlp_colsum(dZ, rows, int(E), gb2d, st, nullptr), "bwd") &&
                  cu.ok(mlp_gemm(dZ, dW2, nullptr, dH, rows, int(H), int(E), 0, 1, 0, 0, 0, st, nullptr), "bwd") &&
                  cu.ok(mlp_relu_backward(dH, Hh, int64_t(rows) * H, st, nullptr), "bwd") &&
                  cu.ok(mlp_gemm(dH, dX, nullptr, g1, int(H), int(d), rows, 1, 1, 0, 0, 0, st, nullptr), "bwd") &&
                  cu.ok(mlp_colsum(dH, rows, int(H), gb1d, st, nullptr), "bwd") && cu.ok(cudaDeviceSynchronize(), "sync");
        if (!ok) rc = SSG_ECUDA;
        if (!rc) {
            cudaMemcpy(loss, stat, 4, cudaMemcpyDeviceToHost);
            cudaMemcpy(gW1, g1, size_t(H) * d * 4, cudaMemcpyDeviceToHost);
            cudaMemcpy(gb1, gb1d, size_t(H) * 4, cudaMemcpyDeviceToHost);
            cudaMemcpy(gW2, g2, size_t(E) * H * 4, cudaMemcpyDeviceToHost);
            cudaMemcpy(gb2, gb2d, size_t(E) * 4, cudaMemcpyDeviceToHost);
        }
    }
    for (float *p : bufs) cudaFree(p);
    if (rc) err = cu.err;
    return rc;
}

}  // namespace ssg
