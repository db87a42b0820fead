"""CPU FP64 reference of the learned shortlist's network -- TEST INFRASTRUCTURE.

Only tests/, the smoke check and the benchmark's CPU legs import this module;
the library never calls it.  The learned shortlist has no counterpart in
SimilaritySearch.jl: the reference's nearest analogue is the exact re-scoring
of a candidate list, rerank! (src/rerank.jl:22-86), whose semantics the
shortlist's last stage keeps.  What is restated here is the published
triplet-loss objective (Schroff et al., FaceNet, 2015) on a two-layer
perceptron, with its gradients derived by hand:

    h = relu(x W1^T + b1)            W1: H x d,  b1: H
    z = h W2^T + b2                  W2: E x H,  b2: E
    l_b = max(0, |z_a - z_p|^2 - |z_a - z_n|^2 + margin)
    L = mean_b l_b

The batch X holds 3B rows: anchors, then positives, then negatives.
"""
from __future__ import annotations

import numpy as np


def forward(W1, b1, W2, b2, X):
    """Hidden pre-activations, hidden activations and embeddings (FP64)."""
    X = np.asarray(X, np.float64)
    pre = X @ np.asarray(W1, np.float64).T + np.asarray(b1, np.float64)
    h = np.maximum(pre, 0.0)
    z = h @ np.asarray(W2, np.float64).T + np.asarray(b2, np.float64)
    return pre, h, z


def triplet_loss_and_grads(W1, b1, W2, b2, X, margin=1.0):
    """Mean triplet loss over the batch and its gradients with respect to
    W1, b1, W2, b2 (all FP64).  Inactive triplets (l_b <= 0) contribute
    nothing, matching the subgradient 0 at the hinge."""
    X = np.asarray(X, np.float64)
    B = X.shape[0] // 3
    pre, h, z = forward(W1, b1, W2, b2, X)
    za, zp, zn = z[:B], z[B:2 * B], z[2 * B:]
    l = ((za - zp) ** 2).sum(1) - ((za - zn) ** 2).sum(1) + margin
    act = (l > 0.0).astype(np.float64)[:, None]
    loss = float(np.maximum(l, 0.0).mean())
    s = 2.0 / B
    dz = np.concatenate([s * act * (zn - zp), -s * act * (za - zp), s * act * (za - zn)])
    gW2 = dz.T @ h
    gb2 = dz.sum(0)
    dh = (dz @ np.asarray(W2, np.float64)) * (pre > 0.0)
    gW1 = dh.T @ X
    gb1 = dh.sum(0)
    return loss, gW1, gb1, gW2, gb2


def embed(W1, b1, W2, b2, X):
    return forward(W1, b1, W2, b2, X)[2]
