"""Writes tests/golden/knn_golden.npz: small seeded k-NN cases with the
results of the oracle (oracle/knn_oracle.c, sequential sums), committed so
the GPU tests compare against fixed vectors as well as the live oracle.

Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


def main():
    rng = np.random.default_rng(20261203)
    out = {}
    float_cases = [("sql2", 500, 16, 20, 10), ("l2", 500, 16, 20, 10), ("normcosine", 400, 24, 20, 7),
                   ("cosine", 400, 24, 20, 7), ("ip", 400, 24, 20, 7)]
    for name, n, d, m, k in float_cases:
        X = rng.standard_normal((n, d), dtype=np.float32)
        Q = rng.standard_normal((m, d), dtype=np.float32)
        if name == "normcosine":
            X /= np.linalg.norm(X, axis=1, keepdims=True)
            Q /= np.linalg.norm(Q, axis=1, keepdims=True)
        ids, dists = O.searchbatch(name, X, Q, k)
        out[f"{name}_X"], out[f"{name}_Q"] = X, Q
        out[f"{name}_ids"], out[f"{name}_dists"] = ids, dists
    # Hamming with heavy ties: 4 words but only the low 3 bits of word 0 vary
    X = np.zeros((1000, 4), dtype=np.uint64)
    X[:, 0] = rng.integers(0, 8, size=1000).astype(np.uint64)
    X[:, 2] = rng.integers(0, 2**63, size=1000, dtype=np.uint64) & np.uint64(0xF)
    Q = X[rng.integers(0, 1000, size=20)].copy()
    ids, dists = O.searchbatch("hamming", X, Q, 16)
    out["hamming_X"], out["hamming_Q"], out["hamming_ids"], out["hamming_dists"] = X, Q, ids, dists
    # allknn (self kept), n=300, dim=6 like test/testparallelexhaustive.jl
    X = rng.random((300, 6), dtype=np.float32)
    ids, dists = O.allknn("sql2", X, 4)
    out["allknn_X"], out["allknn_ids"], out["allknn_dists"] = X, ids, dists
    np.savez_compressed(os.path.join(HERE, "knn_golden.npz"), **out)


if __name__ == "__main__":
    main()
