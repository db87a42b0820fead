"""Pins the FP64 reference of the learned shortlist's network (oracle/
mlp_oracle.py) before the GPU gradients are checked against it: its analytic
gradients agree with central finite differences of its own loss."""
import numpy as np

from oracle import mlp_oracle as MO


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    d, H, E, B = 7, 5, 3, 4
    P = [rng.standard_normal((H, d)), rng.standard_normal(H) * 0.1, rng.standard_normal((E, H)),
         rng.standard_normal(E) * 0.1]
    a = rng.standard_normal((B, d))
    # positives far from their anchors, negatives near: the hinges are active
    X = np.concatenate([a, a + rng.standard_normal((B, d)), a + 0.1 * rng.standard_normal((B, d))])
    loss, *grads = MO.triplet_loss_and_grads(*P, X, margin=3.0)
    assert loss > 0.0
    eps = 1e-6
    for p, g in zip(P, grads):
        num = np.zeros_like(p)
        for i in np.ndindex(p.shape):
            old = p[i]
            p[i] = old + eps
            lp = MO.triplet_loss_and_grads(*P, X, margin=3.0)[0]
            p[i] = old - eps
            lm = MO.triplet_loss_and_grads(*P, X, margin=3.0)[0]
            p[i] = old
            num[i] = (lp - lm) / (2 * eps)
        assert np.allclose(num, g, rtol=1e-5, atol=1e-7)


def test_oracle_inactive_triplets_have_no_gradient():
    rng = np.random.default_rng(1)
    d, H, E, B = 6, 4, 3, 5
    P = [rng.standard_normal((H, d)), np.zeros(H), rng.standard_normal((E, H)), np.zeros(E)]
    a = rng.standard_normal((B, d))
    X = np.concatenate([a, a, a + 100.0])        # positives = anchors, negatives far away
    loss, gW1, gb1, gW2, gb2 = MO.triplet_loss_and_grads(*P, X, margin=1.0)
    assert loss == 0.0
    for g in (gW1, gb1, gW2, gb2):
        assert not np.any(g)
