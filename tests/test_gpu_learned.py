"""GPU tests of the learned shortlist: the hand-written forward / backward
kernels against the FP64 CPU oracle, what the trained network gains over the
same pipeline without it (a random projection), the recall-driven fallback to
the plain method, model files, and the exactness of the returned distances."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_package
from oracle import mlp_oracle as MO
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ss():
    mod = load_package()
    mod.build()
    return mod


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def gpu_grads(ss, W1, b1, W2, b2, X, margin):
    N = ss._native
    H, d = W1.shape
    E = W2.shape[0]
    B = X.shape[0] // 3
    loss = np.zeros(1, np.float32)
    gW1 = np.zeros_like(W1); gb1 = np.zeros_like(b1); gW2 = np.zeros_like(W2); gb2 = np.zeros_like(b2)
    N.check(N.lib().ssg_mlp_grad_check(d, H, E, _ptr(W1), _ptr(b1), _ptr(W2), _ptr(b2), _ptr(X), B,
                                       C.c_float(margin), _ptr(loss), _ptr(gW1), _ptr(gb1), _ptr(gW2), _ptr(gb2)))
    return float(loss[0]), gW1, gb1, gW2, gb2


@pytest.mark.parametrize("d,H,E,B", [(40, 24, 8, 30), (130, 70, 17, 65), (768, 256, 64, 128)])
def test_mlp_gradients_match_fp64_oracle(ss, d, H, E, B):
    rng = np.random.default_rng(d + H + E)
    W1 = (rng.standard_normal((H, d)) * np.sqrt(2.0 / d)).astype(np.float32)
    b1 = (rng.standard_normal(H) * 0.1).astype(np.float32)
    W2 = (rng.standard_normal((E, H)) * np.sqrt(1.0 / H)).astype(np.float32)
    b2 = (rng.standard_normal(E) * 0.1).astype(np.float32)
    X = rng.standard_normal((3 * B, d)).astype(np.float32)
    X[B:2 * B] = X[:B] + 0.5 * X[B:2 * B]
    X[2 * B:] = X[:B] + 0.5 * X[2 * B:]
    # a margin half-way between two neighbouring values of |za-zn|^2 - |za-zp|^2
    # near their median: about half the triplets are active, none at the hinge
    _, _, z = MO.forward(W1, b1, W2, b2, X)
    gap = np.sort(((z[:B] - z[2 * B:]) ** 2).sum(1) - ((z[:B] - z[B:2 * B]) ** 2).sum(1))
    margin = float(0.5 * (gap[B // 2 - 1] + gap[B // 2]))
    loss, gW1, gb1, gW2, gb2 = gpu_grads(ss, W1, b1, W2, b2, X, margin)
    rl, rW1, rb1, rW2, rb2 = MO.triplet_loss_and_grads(W1, b1, W2, b2, X, margin)
    # FP32 accumulation over <= 3B rows (and d terms): relative 1e-4 of the
    # largest gradient entry (hinges exactly at zero are measure-zero here)
    assert abs(loss - rl) <= 1e-4 * max(1.0, abs(rl))
    # b2's gradient vanishes analytically (the anchor, positive and negative
    # gradients of a triplet sum to zero), so its error is measured on the
    # scale of the W2 gradient
    for g, r in ((gW1, rW1), (gb1, rb1), (gW2, rW2), (gb2, rb2)):
        scale = max(np.abs(r).max(), np.abs(rW2).max() if r is rb2 else 0.0)
        assert np.abs(g - r).max() <= 1e-4 * scale


def latent_data(rng, n, d=256, lat=16, noise=1.0, m=300):
    """Points near a random 16-d linear subspace of R^256 with isotropic noise:
    the neighbour structure lives in the subspace, which a trained network can
    find and a random projection cannot."""
    Z = rng.standard_normal((n, lat)).astype(np.float32)
    A = (rng.standard_normal((lat, d)) / np.sqrt(lat)).astype(np.float32)
    X = (Z @ A + rng.standard_normal((n, d)) * (noise * np.sqrt(lat / d))).astype(np.float32)
    Q = (X[rng.integers(0, n, size=m)] + rng.standard_normal((m, d)) * 0.05).astype(np.float32)
    return X, Q


def search(ss, idx, Q, k):
    ids, dists = ss.searchbatch(idx, ss.GenericContext(logger=None), ss.MatrixDatabase.from_rows(Q), k)
    return np.ascontiguousarray(ids.T), np.ascontiguousarray(dists.T)


def make(ss, X, precision="fp32", **params):
    return ss.GPUExhaustiveSearch(ss.Dist.SqL2(), ss.MatrixDatabase.from_rows(X), precision=precision, **params)


def recall_of(ss, X, Q, hidden, S, seed=5):
    idx = make(ss, X)
    idx.set_param("plain", 1)
    gold, _ = search(ss, idx, Q, 10)
    idx.set_param("plain", 0)
    stats = idx.train_mlp(sample=len(X), triplets=200_000, epochs=3, hidden=hidden, out_dim=32, batch=1024,
                          lr=1e-3, seed=seed, target_recall=0.0)
    idx.set_param("shortlist", S)
    ids, dists = search(ss, idx, Q, 10)
    assert idx.get_param("learned_used") == 1
    return O.macrorecall(gold, ids), ids, dists, stats


def test_trained_network_beats_random_projection(ss):
    rng = np.random.default_rng(2024)
    X, Q = latent_data(rng, 20000)
    r_rp, _, _, st_rp = recall_of(ss, X, Q, hidden=0, S=64)
    r_mlp, ids, dists, st = recall_of(ss, X, Q, hidden=128, S=64)
    assert st_rp["train_steps"] == 0 and st["train_steps"] == 3 * ((200_000 + 1023) // 1024)
    assert st["train_loss"] < 0.5
    # the pipeline with the trained network recovers clearly more of the true
    # 10-NN from the same 64-candidate shortlist than with a random projection
    assert r_mlp >= r_rp + 0.08, (r_mlp, r_rp)
    # distances are exact FP32 and rows sorted by (distance, id)
    for j in range(20):
        pairs = [(float(dists[j, t]), int(ids[j, t])) for t in range(10)]
        assert pairs == sorted(pairs)
        for dd, i in pairs:
            assert np.float32(dd) == np.float32(O.evaluate("sql2", X[i - 1], Q[j]))


def test_learned_falls_back_to_plain_below_target(ss):
    rng = np.random.default_rng(77)
    X, Q = latent_data(rng, 6000, m=120)
    idx = make(ss, X)
    plain_ids, plain_d = search(ss, idx, Q, 10)
    idx.train_mlp(sample=6000, triplets=0, epochs=0, hidden=0, out_dim=8, seed=3)
    idx.set_param("shortlist", 12)          # too short for recall 0.99
    assert idx.get_param("learned_ready") == 1
    assert idx.get_param("learned_recall") < 0.99
    ids, dists = search(ss, idx, Q, 10)
    assert idx.get_param("learned_used") == 0
    assert np.array_equal(ids, plain_ids) and np.array_equal(dists, plain_d)
    # with the target lowered the learned path answers
    idx.set_param("learned_target", 0.0)
    ids2, _ = search(ss, idx, Q, 10)
    assert idx.get_param("learned_used") == 1
    # switched off by the caller: plain again
    idx.set_param("learned", 0)
    ids3, d3 = search(ss, idx, Q, 10)
    assert idx.get_param("learned_used") == 0
    assert np.array_equal(ids3, plain_ids) and np.array_equal(d3, plain_d)


def test_learned_full_shortlist_equals_plain(ss):
    rng = np.random.default_rng(5)
    X, Q = latent_data(rng, 700, m=90)
    idx = make(ss, X)
    plain_ids, plain_d = search(ss, idx, Q, 10)
    idx.train_mlp(sample=700, triplets=5000, epochs=2, hidden=64, out_dim=16, batch=256, seed=9)
    idx.set_param("shortlist", 700)        # every object: the rerank sees all
    assert idx.get_param("learned_recall") == 1.0
    ids, dists = search(ss, idx, Q, 10)
    assert idx.get_param("learned_used") == 1
    assert np.array_equal(ids, plain_ids) and np.array_equal(dists, plain_d)
    # appended objects enter the shortlist: a query equal to one of them finds
    # it at distance 0 with its new id
    extra = (rng.standard_normal((50, 256)) * 0.01).astype(np.float32)
    ss.append_items_b(idx, ss.GenericContext(logger=None), ss.MatrixDatabase.from_rows(extra))
    idx.set_param("shortlist", 750)
    ids, dists = search(ss, idx, extra[:5], 3)
    assert idx.get_param("learned_used") == 1
    assert list(ids[:, 0]) == [701, 702, 703, 704, 705] and not np.any(dists[:, 0])


def test_model_file_round_trip(ss, tmp_path):
    rng = np.random.default_rng(8)
    X, Q = latent_data(rng, 5000, m=100)
    a = make(ss, X)
    a.train_mlp(sample=5000, triplets=20000, epochs=2, hidden=64, out_dim=16, batch=512, seed=4, target_recall=0.0)
    a.set_param("shortlist", 100)
    ia, da = search(ss, a, Q, 10)
    path = tmp_path / "model.ssgmlp"
    a.save_model(str(path))
    raw = path.read_bytes()
    assert raw[:8] == b"SSGMLP01"
    d, H, E = np.frombuffer(raw[8:32], "<i8")
    assert (d, H, E) == (256, 64, 16)
    assert len(raw) == 32 + 4 * (H * d + H + E * H + E)
    b = make(ss, X, learned_target=0.0)
    b.load_model(str(path))
    b.set_param("shortlist", 100)
    ib, db = search(ss, b, Q, 10)
    assert b.get_param("learned_used") == 1
    assert np.array_equal(ia, ib) and np.array_equal(da, db)
    # a model for another dimension is refused
    c = make(ss, X[:, :128].copy())
    with pytest.raises(ss.ArgumentError):
        c.load_model(str(path))


def test_train_argument_errors(ss):
    rng = np.random.default_rng(1)
    X, _ = latent_data(rng, 200, m=1)
    idx = make(ss, X)
    with pytest.raises(ss.ArgumentError):
        idx.train_mlp(sample=5)
    with pytest.raises(ss.ArgumentError):
        idx.train_mlp(out_dim=0)
    with pytest.raises(ss.ArgumentError):
        idx.set_param("shortlist", 64)       # no model yet
    with pytest.raises(ss.ArgumentError):
        idx.set_param("learned_target", 1.5)
    sk = ss.GPUExhaustiveSearch(ss.Dist.Bits.Hamming(), ss.MatrixDatabase.from_rows(
        rng.integers(0, 2**63, size=(64, 2), dtype=np.uint64)))
    with pytest.raises(ss._native.UnsupportedError):
        sk.train_mlp(sample=64)
